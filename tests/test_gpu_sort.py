"""cudiv::Sort (stable key/value sort) against numpy's stable argsort,
including empty input, one element, one huge cube and large key ranges."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sort(keys, vals):
    import torch
    from gpucell_gb300 import _lib
    k = torch.as_tensor(keys.astype(np.int32), device="cuda")
    v = torch.as_tensor(vals.astype(np.int32), device="cuda")
    _lib.call("gc_cudiv_Sort", int(keys.size), C.c_void_p(k.data_ptr() if keys.size else 0),
              C.c_void_p(v.data_ptr() if keys.size else 0))
    torch.cuda.synchronize()
    return k.cpu().numpy(), v.cpu().numpy()


@pytest.mark.parametrize("n,K", [(0, 10), (1, 1), (1000, 1), (5000, 7), (100000, 3000), (1 << 20, 150000)])
def test_sort_matches_stable_argsort(cuda_device, n, K):
    from gpucell_gb300 import _lib
    _lib.call("gc_shutdown")            # no grid: the key range is found on the device
    rng = np.random.default_rng(n + K)
    keys = rng.integers(0, K, size=n).astype(np.int32)
    vals = rng.permutation(n).astype(np.int32)
    if n == 0:
        _lib.call("gc_cudiv_Sort", 0, C.c_void_p(0), C.c_void_p(0))
        return
    ks, vs = _sort(keys, vals)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(ks, keys[order])
    assert np.array_equal(vs, vals[order])
