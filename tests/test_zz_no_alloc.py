"""hrt_sort_morton_pairs_noalloc: the LBVH's pair sort for callers that cannot
call cudaMalloc (hosts whose device memory belongs to another allocator that
reserves it up front, latency-bound paths that cannot take an allocation's
synchronisation).  Its scratch is a fixed device array inside the library, so
the test checks that two calls in a row -- the second one finding the first
call's leftovers in that array -- both give exactly the order the regular
build (hrt_add_geom_triangles3f) produced, and that a call leaves the device's
free memory and torch's allocator untouched.

This file is collected last on purpose: a run that stops at the first failure
has already run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _entry():
    from heavyrt_gb300 import engine as E

    f = E.lib().hrt_sort_morton_pairs_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]
    return f


def _sorted_by_existing_entry_point(n_tris, seed):
    """Morton pairs before and after the sort of a regular geometry build."""
    from heavyrt_gb300 import SceneRT
    from heavyrt_gb300 import engine as E
    from heavyrt_gb300 import workload as wl

    v, idx = wl.soup(seed, n_tris)
    s = SceneRT()
    gid = s.AddGeom_Triangles3f(v, v.shape[0], idx, idx.size, vByteStride=16)
    unsorted = s.export(gid, E.EXPORT_MORTON_UNSORTED).reshape(-1, 2)
    want = s.export(gid, E.EXPORT_MORTON_SORTED).reshape(-1, 2)
    s.close()
    return unsorted, want


def test_noalloc_sort_matches_build_sort_twice(native):
    import torch

    from heavyrt_gb300 import engine as E

    sort = _entry()
    stream = torch.cuda.current_stream().cuda_stream
    # the second input is smaller, so it runs over the first call's leftover scratch
    for n_tris, seed in ((200_000, 11), (70_001, 12)):
        unsorted, want = _sorted_by_existing_entry_point(n_tris, seed)
        keys = torch.from_numpy(unsorted[:, 0].astype(np.uint32).view(np.int32)).cuda()
        vals = torch.from_numpy(unsorted[:, 1].astype(np.uint32).view(np.int32)).cuda()
        torch.cuda.synchronize()
        st = sort(C.c_void_p(keys.data_ptr()), C.c_void_p(vals.data_ptr()), n_tris, C.c_void_p(stream))
        assert st == E.HRT_OK
        got = np.stack([keys.cpu().numpy().view(np.uint32), vals.cpu().numpy().view(np.uint32)], axis=1)
        np.testing.assert_array_equal(got, want)  # integer data: bit-exact


def test_noalloc_sort_allocates_nothing(native):
    """A warm call changes neither the device's free memory nor torch's
    allocator: the scratch is the library's fixed array."""
    import torch

    from heavyrt_gb300 import engine as E

    sort = _entry()
    stream = torch.cuda.current_stream().cuda_stream
    unsorted, want = _sorted_by_existing_entry_point(100_000, 13)
    keys = torch.from_numpy(unsorted[:, 0].astype(np.uint32).view(np.int32)).cuda()
    vals = torch.from_numpy(unsorted[:, 1].astype(np.uint32).view(np.int32)).cuda()
    k0, v0 = keys.clone(), vals.clone()
    assert sort(C.c_void_p(keys.data_ptr()), C.c_void_p(vals.data_ptr()), keys.numel(), C.c_void_p(stream)) == E.HRT_OK
    keys.copy_(k0)
    vals.copy_(v0)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0 = torch.cuda.memory_allocated()
    assert sort(C.c_void_p(keys.data_ptr()), C.c_void_p(vals.data_ptr()), keys.numel(), C.c_void_p(stream)) == E.HRT_OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_allocated() == alloc0
    got = np.stack([keys.cpu().numpy().view(np.uint32), vals.cpu().numpy().view(np.uint32)], axis=1)
    np.testing.assert_array_equal(got, want)


def test_noalloc_sort_rejects_oversize(native):
    from heavyrt_gb300 import engine as E

    sort = _entry()
    big = (1 << 18) + 1
    assert sort(C.c_void_p(16), C.c_void_p(16), big, None) == E.HRT_ERR_CAPACITY
    assert sort(None, None, 5, None) == E.HRT_ERR_INVALID_ARGUMENT
