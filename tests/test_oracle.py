"""The oracle (C restatement of HeavyRT's LBVH build + BVH2CommonRT traversal)
against the golden vectors produced by HeavyRT's own code, and against that
code live where its sources are present.  CPU only."""
import numpy as np
import pytest

from conftest import GOLDEN, golden_cases


def _load(case):
    return dict(np.load(GOLDEN / f"golden_{case}.npz"))


@pytest.mark.parametrize("case", golden_cases())
def test_oracle_build_matches_golden(host_libs, case):
    from oracle import oracle as orc

    g = _load(case)
    o = orc.OracleBVH(g["verts"], g["idx"])
    assert o.status == 0
    np.testing.assert_array_equal(o.scene_box().view(np.uint32), g["scene_box"].view(np.uint32))
    np.testing.assert_array_equal(o.morton_unsorted(), g["morton_unsorted"])
    np.testing.assert_array_equal(o.morton_sorted(), g["morton_sorted"])
    np.testing.assert_array_equal(o.compressed(), g["compressed"])
    np.testing.assert_array_equal(o.run_starts(), g["run_starts"])
    np.testing.assert_array_equal(o.lr_nodes().view(np.uint32), g["lr_nodes"])
    np.testing.assert_array_equal(o.lr_counts(), g["lr_counts"])
    np.testing.assert_array_equal(o.peach_nodes().view(np.uint32), g["peach_nodes"])
    np.testing.assert_array_equal(o.prim_indices(), g["prim_indices"])
    np.testing.assert_array_equal(o.sorted_indices(), g["sorted_indices"])


@pytest.mark.parametrize("case", golden_cases())
def test_oracle_trace_matches_golden(host_libs, case):
    from oracle import oracle as orc

    g = _load(case)
    o = orc.OracleBVH(g["verts"], g["idx"])
    hits, (pairs, tris), _ = o.trace(g["rays"], counters=True, threads=1)
    np.testing.assert_array_equal(hits.view(np.uint32).reshape(-1, 8), g["hits"].reshape(-1, 8))
    anyh = o.trace(g["rays"], any_hit=True)
    np.testing.assert_array_equal(anyh, g["any"])
    # HeavyRT's own counters (core/BVH2CommonRT.cpp:68-69,125): 2 nodes per pair, BLB = 64 B/pair + 60 B/triangle
    n = g["rays"].shape[0]
    avg_nc, avg_tc, avg_blb = g["ref_counters"]
    assert abs(2.0 * pairs / n - avg_nc) < 1e-3
    assert abs(tris / n - avg_tc) < 1e-3
    assert abs((64.0 * pairs + 60.0 * tris) / n - avg_blb) < 1e-2


def test_anyhit_is_nearest_found(host_libs):
    """Any-hit semantics (HeavyRT siblings, core/BVH2CommonRTStacklessLBVH.cpp:161-165):
    true exactly when the nearest-hit traversal accepts some triangle."""
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    v, idx, _ = wl.heightfield(11, 48, 48)
    rays = np.concatenate([wl.rays_at_triangles(5, v, idx, 4000, jitter=0.05), wl.sphere_rays(6, 4000)])
    rays[::3, 7] = 0.05  # short rays: some hits fall beyond tFar
    o = orc.OracleBVH(v, idx)
    hits = o.trace(rays)
    anyh = o.trace(rays, any_hit=True)
    np.testing.assert_array_equal(anyh, hits["geomId"] != 0xFFFFFFFF)


def test_oracle_flags_leaf_overflow(host_libs):
    """More than 127 triangles with one Morton code overflow the reference's
    7-bit leaf count (core/raytrace_common.h:40,48-51); the oracle flags it."""
    from oracle import oracle as orc

    tri = np.array([[0, 0, 0, 1], [1, 0, 0, 1], [0, 1, 0, 1]], dtype=np.float32)
    v = np.concatenate([tri] * 200 + [tri + np.array([5, 5, 5, 0], np.float32)])
    idx = np.arange(v.shape[0], dtype=np.uint32)
    o = orc.OracleBVH(v, idx)
    assert o.status == 1


REF_CASES = [("soup", 2), ("soup", 17), ("soup", 4096), ("soup", 9000), ("soup", 30000), ("hf", 32), ("hf", 128)]


@pytest.mark.parametrize("kind,n", REF_CASES)
def test_oracle_matches_reference_live(host_libs, kind, n):
    """Bit-exact against the reference's own builder and traversal, compiled
    from its sources (skipped where they are absent)."""
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    if orc.reference_harness() is None:
        pytest.skip("reference sources not present on this machine")
    if kind == "soup":
        v, idx = wl.soup(300 + n, n)
    else:
        v, idx, _ = wl.heightfield(300 + n, n, n)
    rays = np.concatenate([wl.rays_at_triangles(n, v, idx, 2000, jitter=0.02), wl.sphere_rays(n, 500)])
    ref = orc.run_reference(v, idx, rays)
    o = orc.OracleBVH(v, idx)
    np.testing.assert_array_equal(o.morton_unsorted(), ref["morton_unsorted"])
    np.testing.assert_array_equal(o.morton_sorted(), ref["morton_sorted"])
    np.testing.assert_array_equal(o.lr_nodes().view(np.uint32), ref["lr_nodes"].view(np.uint32))
    np.testing.assert_array_equal(o.lr_counts(), ref["lr_counts"])
    np.testing.assert_array_equal(o.peach_nodes().view(np.uint32), ref["peach_nodes"].view(np.uint32))
    np.testing.assert_array_equal(o.prim_indices(), ref["prim_indices"])
    np.testing.assert_array_equal(o.trace(rays).view(np.uint32), ref["hits"].view(np.uint32))
    np.testing.assert_array_equal(o.trace(rays, any_hit=True), ref["any"])


def _eye_cases():
    z = np.load(GOLDEN / "raygen_eye.npz")
    k = 0
    while f"rays{k}" in z:
        yield (z[f"proj_inv{k}"], z[f"world_view_inv{k}"], *[int(x) for x in z[f"size{k}"]],
               *[float(x) for x in z[f"range{k}"]], z[f"rays{k}"])
        k += 1


def test_eye_rays_restatement_matches_reference_fixture(host_libs):
    """The renderers' eye-ray set-up restated in C equals the reference's own
    helpers (examples/render_common.h, compiled against the LiteMath stand-in)."""
    from oracle import oracle as orc

    for p, v, w, h, tn, tf, want in _eye_cases():
        got = orc.eye_rays(p, v, w, h, tn, tf)
        np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
        live = orc.reference_eye_rays(p, v, w, h, tn, tf)
        if live is not None:
            np.testing.assert_array_equal(live.view(np.uint32), want.view(np.uint32))


def _render_fixture():
    return dict(np.load(GOLDEN / "render_frames.npz"))


def _render_case(z, k):
    w, h, r = (int(x) for x in z[f"{k}_params"])
    zn, zf, rad, pw = (float(x) for x in z[f"{k}_fparams"])
    return dict(proj_inv=z[f"{k}_proj_inv"], world_view_inv=z[f"{k}_world_view_inv"], width=w, height=h, z_near=zn,
                z_far=zf, rays_per_pixel=r, radius=rad, power=pw, norm_matrix=z[f"{k}_norm_matrix"])


def test_qmc_tile_restatement_matches_reference_fixture(host_libs):
    """RTAO's quasi-random sample tile: the generator's direction table and the
    binned tile equal the reference's (core/common/qmc_sobol_niederreiter.cpp,
    examples/02_rtao/rtao_host.cpp:383-414)."""
    import hashlib

    from oracle import oracle as orc

    z = _render_fixture()
    np.testing.assert_array_equal(orc.qmc_table(), z["qmc_table"])
    for r in (1, 3, 4, 16):
        digest = np.frombuffer(hashlib.sha256(orc.rtao_tile(r).tobytes()).digest(), np.uint8)
        np.testing.assert_array_equal(digest, z[f"tile_sha256_r{r}"])


def test_render_frames_restatement_matches_reference_fixture(host_libs):
    """The example renderers' frames restated in C (eye-ray renderer: packed order
    and palette; RTAO: hit points with packed normals, AO rays, occlusion,
    visibility, colours) equal the reference's own kernels on both fixture frames."""
    from oracle import oracle as orc

    z = _render_fixture()
    b = orc.OracleBVH(z["verts"], z["idx"])
    for k in ("a", "b"):
        c = _render_case(z, k)
        o = orc.rtao_frame(b, z["verts"], z["normals"], c["proj_inv"], c["world_view_inv"], c["width"], c["height"],
                           c["z_near"], c["z_far"], c["rays_per_pixel"], c["radius"], c["power"], c["norm_matrix"])
        np.testing.assert_array_equal(o["positions"].view(np.uint32), z[f"{k}_positions"].view(np.uint32))
        np.testing.assert_array_equal(o["ao_rays"][o["ao_valid"]].view(np.uint32), z[f"{k}_ao_rays"].view(np.uint32))
        np.testing.assert_array_equal(o["ao_hit"][o["ao_valid"]], z[f"{k}_ao_hit"])
        np.testing.assert_array_equal(o["visibility"].view(np.uint32), z[f"{k}_visibility"].view(np.uint32))
        np.testing.assert_array_equal(o["colors"], z[f"{k}_colors"])
        assert 0 < o["ao_valid"].mean() < 1 and 0 < z[f"{k}_ao_hit"].mean() < 1
        if f"{k}_eye_packed" in z:
            np.testing.assert_array_equal(orc.pack_xy(c["width"], c["height"]), z[f"{k}_eye_packed"])
            np.testing.assert_array_equal(orc.eye_frame(b, c["proj_inv"], c["world_view_inv"], c["width"], c["height"]),
                                          z[f"{k}_eye_colors"])


def test_render_frames_match_reference_live(host_libs):
    """Where the reference sources are present: a fresh frame of each renderer
    (another camera, 8 samples) from the reference's own kernels equals the
    restatement."""
    from oracle import oracle as orc

    z = _render_fixture()
    c = _render_case(z, "a")
    v, idx, nrm = z["verts"], z["idx"], z["normals"]
    wv = np.linalg.inv(np.asarray(np.linalg.inv(c["world_view_inv"]), np.float64) @
                       np.array([[0.96, -0.28, 0, 0.05], [0.28, 0.96, 0, 0], [0, 0, 1, 0.02], [0, 0, 0, 1]]))
    wv = wv.astype(np.float32)
    ref = orc.reference_render("rtao", v, idx, c["proj_inv"], wv, 40, 32, normals=nrm, rays_per_pixel=8, radius=0.25)
    if ref is None:
        pytest.skip("reference sources absent")
    b = orc.OracleBVH(v, idx)
    o = orc.rtao_frame(b, v, nrm, c["proj_inv"], wv, 40, 32, 0.0, 3.4028234663852886e38, 8, 0.25)
    hit = o["positions"][:, 1] < orc.AO_HIT_BACK
    np.testing.assert_array_equal(o["positions"].view(np.uint32), ref["positions"].view(np.uint32))
    np.testing.assert_array_equal(o["ao_rays"].view(np.uint32), ref["ao_rays"].view(np.uint32))
    np.testing.assert_array_equal(o["ao_hit"], ref["ao_hit"])
    np.testing.assert_array_equal(o["visibility"][hit], ref["visibility"][hit])
    np.testing.assert_array_equal(o["colors"], ref["colors"])
    e = orc.reference_render("eye", v, idx, c["proj_inv"], wv, 40, 32)
    np.testing.assert_array_equal(orc.eye_frame(b, c["proj_inv"], wv, 40, 32), e["colors"])
    np.testing.assert_array_equal(orc.pack_xy(40, 32), e["packed"])


def _bary64(rays, verts, tri_idx):
    """FP64 barycentrics (w_A, w_B, w_C) and t of each ray against one
    triangle (vertex indices per ray, [n, 3])."""
    v = np.asarray(verts, np.float64)[:, :3]
    a, b, c = v[tri_idx[:, 0]], v[tri_idx[:, 1]], v[tri_idx[:, 2]]
    o, d = rays[:, 0:3].astype(np.float64), rays[:, 4:7].astype(np.float64)
    e1, e2 = b - a, c - a
    p = np.cross(d, e2)
    det = np.einsum("ij,ij->i", e1, p)
    s = o - a
    q = np.cross(s, e1)
    wb = np.einsum("ij,ij->i", s, p) / det
    wc = np.einsum("ij,ij->i", d, q) / det
    t = np.einsum("ij,ij->i", e2, q) / det
    return np.stack([1 - wb - wc, wb, wc], axis=1), t


def test_oracle_watertight_heightfield_edges_never_leak(host_libs):
    """The watertight restatement on a closed heightfield: vertical rays aimed
    exactly at every interior grid vertex and edge midpoint all hit."""
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    nx = 64
    v, idx, _ = wl.heightfield(77, nx, nx)
    xy = v[:, :2].reshape(nx + 1, nx + 1, 2)
    p = np.concatenate([xy.reshape(-1, 2), (0.5 * (xy[:, 1:] + xy[:, :-1])).reshape(-1, 2),
                        (0.5 * (xy[1:, :] + xy[:-1, :])).reshape(-1, 2),
                        (0.5 * (xy[1:, 1:] + xy[:-1, :-1])).reshape(-1, 2)]).astype(np.float32)
    p = p[(np.abs(p) < 1.0).all(axis=1)]
    rays = np.zeros((p.shape[0], 8), np.float32)
    rays[:, 0:2], rays[:, 2], rays[:, 6], rays[:, 7] = p, 3.0, -1.0, 1e9
    o = orc.OracleBVH(v, idx)
    wt = o.trace(rays, watertight=True)
    assert np.all(wt["geomId"] != 0xFFFFFFFF)
    assert o.trace(rays, any_hit=True, watertight=True).all()


def test_oracle_watertight_agrees_with_mt_away_from_edges(host_libs):
    """Away from triangle edges (every FP64 barycentric above 1e-4) the
    watertight test and the reference's MT test hit the same triangle at t
    within 1e-5 relative; against an FP64 evaluation the watertight t is within
    1e-5 relative and its barycentrics within 1e-4 (tighter than MT's on the
    same rays); every watertight hit lies inside its triangle up to FP32
    rounding."""
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    v, idx = wl.soup(21, 20000, off=0.05)
    rays = np.concatenate([wl.rays_at_triangles(3, v, idx, 20000, jitter=0.03), wl.sphere_rays(4, 5000)])
    o = orc.OracleBVH(v, idx)
    mt = o.trace(rays)
    wt = o.trace(rays, watertight=True)
    si = o.sorted_indices().reshape(-1, 3)
    hw = wt["geomId"] != 0xFFFFFFFF
    assert hw.mean() > 0.5
    bw, tw = _bary64(rays[hw], v, si[wt["primId"][hw]])
    assert np.all(bw.min(axis=1) > -1e-5)  # the sheared FP32 vertices stand in for the exact ones
    hm = mt["geomId"] != 0xFFFFFFFF
    both = hm & hw
    bm, _ = _bary64(rays[both], v, si[mt["primId"][both]])
    bw2, _ = _bary64(rays[both], v, si[wt["primId"][both]])
    clear = (bm.min(axis=1) > 1e-4) & (bw2.min(axis=1) > 1e-4)
    assert clear.mean() > 0.9
    np.testing.assert_array_equal(mt["primId"][both][clear], wt["primId"][both][clear])
    tm, tw2 = mt["t"][both][clear].astype(np.float64), wt["t"][both][clear].astype(np.float64)
    assert np.all(np.abs(tm - tw2) <= 1e-5 * np.abs(tm))
    same = wt["primId"][both] == mt["primId"][both]
    b64, t64 = _bary64(rays[both][same], v, si[wt["primId"][both][same]])
    err_w = np.abs(wt["coords"][both][same][:, :2] - b64[:, [2, 1]]).max()  # coords = (w_C, w_B)
    err_m = np.abs(mt["coords"][both][same][:, :2] - b64[:, [2, 1]]).max()
    assert err_w < 1e-4 and err_w <= err_m
    assert np.all(np.abs(wt["t"][both][same] - t64) <= 1e-5 * np.abs(t64))
    # hit/miss differs only for rays near an edge of the triangle one test hit
    only = hm ^ hw
    if only.any():
        prim = np.where(hm[only], mt["primId"][only], wt["primId"][only])
        b, _ = _bary64(rays[only], v, si[prim])
        assert np.all(np.abs(b).min(axis=1) < 1e-5)


def _collapse_walk(nodes, n_tris, run_starts):
    """Walks 4-wide nodes from node 0: every node reached once, the leaf
    starts reached, and the deepest 4-wide level."""
    from oracle import oracle as orc

    seen, starts, depth = set(), [], 0
    stack = [(0, 1)]
    while stack:
        n, d = stack.pop()
        assert n not in seen
        seen.add(n)
        depth = max(depth, d)
        for ref in nodes[n, 24:28]:
            ref = int(ref)
            if ref == orc.EMPTY_REF:
                continue
            if ref & orc.LEAF_BIT:
                starts.append(ref & ~orc.LEAF_BIT)
            else:
                stack.append((ref, d + 1))
    return seen, sorted(starts), depth


@pytest.mark.parametrize("merge", [0, 1, 4])
def test_collapse4_rules_cover_every_run(host_libs, merge):
    """Both collapse rules of the 4-wide restatement reach every node once and
    start a leaf at run starts only, every run start once when nothing merges;
    the even-depth rule's nodes are the internal nodes at even depth; child
    boxes lie inside the box of their slot in the parent."""
    from heavyrt_gb300 import workload as wl
    from oracle import oracle as orc

    hv, hidx, _ = wl.heightfield(5, 40, 30)
    sv, sidx = wl.soup(6, 3000, off=0.05)
    for v, idx in ((hv, hidx), (sv, sidx), (sv[:3], sidx[:3]), (sv[:12], sidx[:6])):
        o = orc.OracleBVH(v, idx)
        lr, cnt, rs = o.lr_nodes(), o.lr_counts(), o.run_starts()
        out = {}
        for rule in (orc.COLLAPSE_EVEN_DEPTH, orc.COLLAPSE_LARGEST_FIRST):
            nodes = orc.collapse4(lr, cnt, rs, o.n_tris, merge, rule)
            seen, starts, depth = _collapse_walk(nodes, o.n_tris, rs)
            assert seen == set(range(len(nodes)))
            assert set(starts) <= set(int(x) for x in rs) and len(set(starts)) == len(starts)
            if merge == 1:
                assert starts == sorted(int(x) for x in rs)
            # slot boxes of a child node enclose nothing outside the parent's slot box
            for n in range(len(nodes)):
                box = nodes[n, 0:24].view(np.float32).reshape(6, 4)
                for k, ref in enumerate(nodes[n, 24:28]):
                    ref = int(ref)
                    if ref == orc.EMPTY_REF or ref & orc.LEAF_BIT:
                        continue
                    cb = nodes[ref, 0:24].view(np.float32).reshape(6, 4)
                    used = nodes[ref, 24:28] != orc.EMPTY_REF
                    assert np.all(cb[0:3, used] >= box[0:3, k:k + 1]) and np.all(cb[3:6, used] <= box[3:6, k:k + 1])
            out[rule] = (len(nodes), depth)
        if o.n_leaves > 1 and merge == 1:
            left, right = lr["leftOffset"].astype(int), lr["escapeIndex"].astype(int)
            L = o.n_leaves
            even, stack = 0, [(0, 0)]
            while stack:
                n, d = stack.pop()
                even += d % 2 == 0
                stack += [(c, d + 1) for c in (left[n], right[n]) if c < L - 1]
            assert out[orc.COLLAPSE_EVEN_DEPTH][0] == even
        o.close()
