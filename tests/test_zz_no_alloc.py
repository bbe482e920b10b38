"""gc_cudiv_Sort_noalloc: the neighbour-grid sort for callers that cannot
let the library allocate device memory (a host program that reserves the
device memory it uses up front, a process under a fixed memory cap, a loop
that must not stall on cudaFree).

It must give exactly the output of gc_cudiv_Sort -- a stable key/value sort
of integers, so the tolerance is bit-exact -- on calls made one after the
other, which share its fixed scratch array; it must leave the library's own
scratch empty and the device's free memory unchanged; and a key outside the
cube range must be reported through gc_device_status, as gc_cudiv_Sort
reports it.  This file is collected last so that a run stopping at the first
failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GC_FLAG_BAD_INDEX = 2


def _sorted_by(name, keys, vals):
    import torch
    from gpucell_gb300 import _lib
    k = torch.as_tensor(keys, device="cuda")
    v = torch.as_tensor(vals, device="cuda")
    _lib.call(name, int(keys.size), C.c_void_p(k.data_ptr()), C.c_void_p(v.data_ptr()))
    torch.cuda.synchronize()
    return k.cpu().numpy(), v.cpu().numpy()


def _scratch_bytes():
    from gpucell_gb300 import _lib
    b = C.c_ulonglong(0)
    _lib.call("gc_scratch_bytes", C.byref(b))
    return int(b.value)


def test_noalloc_sort_matches_sort_on_consecutive_calls(cuda_device):
    from gpucell_gb300 import _lib
    _lib.call("gc_shutdown")     # no grid from earlier tests: both sorts find the key range on the device
    rng = np.random.default_rng(2024)
    cases = [(200000, 50000), (262144, 262144), (1000, 1), (77777, 3)]
    for n, K in cases:
        keys = rng.integers(0, K, size=n).astype(np.int32)
        vals = rng.permutation(n).astype(np.int32)
        want_k, want_v = _sorted_by("gc_cudiv_Sort", keys, vals)
        got_k, got_v = _sorted_by("gc_cudiv_Sort_noalloc", keys, vals)
        assert np.array_equal(got_k, want_k), (n, K)
        assert np.array_equal(got_v, want_v), (n, K)
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(got_v, vals[order])
    assert _lib.device_status() == 0


def test_noalloc_sort_allocates_nothing(cuda_device):
    """After gc_shutdown the library holds no scratch; two no-allocation
    sorts in a row (after one warm-up call, which commits the library's fixed
    array on this device) leave it so and take no device memory."""
    import torch
    from gpucell_gb300 import _lib
    rng = np.random.default_rng(7)
    keys = rng.integers(0, 4096, size=100000).astype(np.int32)
    vals = np.arange(keys.size, dtype=np.int32)
    k = torch.as_tensor(keys, device="cuda")
    v = torch.as_tensor(vals, device="cuda")
    torch.cuda.synchronize()
    _lib.call("gc_shutdown")
    assert _scratch_bytes() == 0
    _lib.call("gc_cudiv_Sort_noalloc", int(keys.size), C.c_void_p(k.data_ptr()), C.c_void_p(v.data_ptr()))
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        k.copy_(torch.as_tensor(keys))
        v.copy_(torch.as_tensor(vals))
        _lib.call("gc_cudiv_Sort_noalloc", int(keys.size), C.c_void_p(k.data_ptr()), C.c_void_p(v.data_ptr()))
        torch.cuda.synchronize()
        assert np.array_equal(v.cpu().numpy(), vals[np.argsort(keys, kind="stable")])
    free1, _ = torch.cuda.mem_get_info()
    assert _scratch_bytes() == 0
    assert free1 == free0, (free0, free1)


def test_noalloc_sort_reports_out_of_range_keys(cuda_device):
    """A negative key, and a key at or beyond the cube count of the grid the
    latest PreConList set, raise GC_FLAG_BAD_INDEX (as gc_cudiv_Sort does)
    instead of being clamped silently; a clean call afterwards reports
    nothing."""
    import torch
    from gpucell_gb300 import _lib
    from gpucell_gb300 import generator as gen
    from gpucell_gb300.host import ParticleSystem
    _lib.call("gc_shutdown")
    assert _lib.device_status() == 0
    keys = np.array([3, -5, 1, 2, 0], np.int32)
    _sorted_by("gc_cudiv_Sort_noalloc", keys, np.arange(5, dtype=np.int32))
    assert _lib.device_status() & GC_FLAG_BAD_INDEX
    assert _lib.device_status() == 0          # read and cleared
    # a grid set by the boundary path's PreConList: keys must lie below its cube count
    cfg = gen.small_channel()
    ps = ParticleSystem(cfg, noise=False)
    ps.update()
    torch.cuda.synchronize()
    assert _lib.device_status() == 0
    ncube = int(ps.size_cube)
    keys = np.array([0, ncube + 7, 1], np.int32)
    _sorted_by("gc_cudiv_Sort_noalloc", keys, np.arange(3, dtype=np.int32))
    assert _lib.device_status() & GC_FLAG_BAD_INDEX
    keys = np.array([2, 0, 1], np.int32)
    got_k, got_v = _sorted_by("gc_cudiv_Sort_noalloc", keys, np.arange(3, dtype=np.int32))
    assert list(got_v) == [1, 2, 0] and _lib.device_status() == 0
    del ps
    _lib.call("gc_shutdown")


def test_noalloc_sort_rejects_oversized_input(cuda_device):
    from gpucell_gb300 import _lib
    lib = _lib.load()
    n = 262144 + 1
    rc = lib.gc_cudiv_Sort_noalloc(n, C.c_void_p(0), C.c_void_p(0))
    assert rc == -1
    assert b"exceeds the fixed scratch" in lib.gc_last_error()
    import torch
    keys = torch.full((10,), 300000, dtype=torch.int32, device="cuda")
    vals = torch.arange(10, dtype=torch.int32, device="cuda")
    _lib.call("gc_shutdown")
    rc = lib.gc_cudiv_Sort_noalloc(10, C.c_void_p(keys.data_ptr()), C.c_void_p(vals.data_ptr()))
    assert rc == -1
    assert b"keys exceed the fixed scratch" in lib.gc_last_error()
