"""gc_cudiv_Sort_noalloc: the neighbour-grid sort for callers that cannot
let the library allocate device memory (a host program that reserves the
device memory it uses up front, a process under a fixed memory cap, a loop
that must not stall on cudaFree).

It must give exactly the output of gc_cudiv_Sort -- a stable key/value sort
of integers, so the tolerance is bit-exact -- on calls made one after the
other, which share its fixed scratch array.  This file is collected last so
that a run stopping at the first failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sorted_by(name, keys, vals):
    import torch
    from gpucell_gb300 import _lib
    k = torch.as_tensor(keys, device="cuda")
    v = torch.as_tensor(vals, device="cuda")
    _lib.call(name, int(keys.size), C.c_void_p(k.data_ptr()), C.c_void_p(v.data_ptr()))
    torch.cuda.synchronize()
    return k.cpu().numpy(), v.cpu().numpy()


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
