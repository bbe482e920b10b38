"""Rouleau labelling from contact pairs through the library's host code
(gc_rouleaux_from_pairs); the GPU search for the pairs is
``FusedSystem.rouleaux`` / ``Ensemble.rouleaux``."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


def from_pairs(ncell: int, pairs) -> tuple[np.ndarray, np.ndarray]:
    """(label per cell, cells per rouleau) for cells 0..ncell-1 joined by
    the (k, 2) contact pairs; rouleaux are numbered by their lowest cell."""
    p = np.ascontiguousarray(np.asarray(pairs, np.int32).reshape(-1, 2))
    label = np.zeros(max(ncell, 1), np.int32)
    size = np.zeros(max(ncell, 1), np.int32)
    n = C.c_int()
    _lib.call("gc_rouleaux_from_pairs", int(ncell), int(p.shape[0]), p.ctypes.data_as(C.c_void_p),
              label.ctypes.data_as(C.c_void_p), size.ctypes.data_as(C.c_void_p), C.byref(n))
    return label[:ncell], size[:n.value]
