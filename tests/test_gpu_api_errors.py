"""The fused C API refuses bad input and calls out of order with a status
code and a message, and leaves the library usable: boxes that are empty or
too short for the cut-off, periodic masks out of range, systems without
particles, options out of range, membrane topologies with indices outside
their arrays, NULL arrays, stepping before set-up, set-up before the state
is loaded, a second set-up, cells after set-up, a negative step count, a
system index out of range, and a rouleau contact distance that is not
positive.  A valid system afterwards still steps."""
import ctypes as C
import dataclasses

import numpy as np
import pytest

from gpucell_gb300 import _lib
from gpucell_gb300 import generator as gen
from gpucell_gb300.fused import FusedSystem, _cell_arrays, _options, _ptr

pytestmark = pytest.mark.gpu


def _create(cfg, bbox=None, pmask=None, opt=None):
    h = C.c_void_p()
    consts = _lib.Structconst(**cfg.consts())
    bb = np.ascontiguousarray(cfg.bbox if bbox is None else bbox, np.float32)
    o = opt or _options(0.1, 128, 0, True, False)
    _lib.call("gc_fused_create", C.byref(consts), _ptr(bb), cfg.pmask if pmask is None else pmask, 0, C.byref(o),
              C.byref(h))
    return h


def _destroy(h):
    if h:
        _lib.call("gc_fused_destroy", h)


def test_bad_create_arguments(cuda_device):
    cfg = gen.small_channel()
    with pytest.raises(_lib.GcError, match="empty or not finite"):
        _create(cfg, bbox=[0, 0, -2, 2, -2, 2])
    with pytest.raises(_lib.GcError, match="periodic axis"):
        _create(cfg, bbox=[0, 1.5, -2, 2, -2, 2])           # x periodic and shorter than 3 cut-offs
    with pytest.raises(_lib.GcError, match="periodic mask"):
        _create(cfg, pmask=9)
    for bad in (_options(2.0, 128, 0, True, False), _options(0.1, 100, 0, True, False)):
        with pytest.raises(_lib.GcError, match="skin|block"):
            _create(cfg, opt=bad)
    empty = dataclasses.replace(cfg, coor=cfg.coor[:0], velhalf=cfg.velhalf[:0], n_b1=0, n_b2=0, n_fluid=0,
                                ncell=0, tri=None, edge=None, betri=None, celltab=None, npar=None, ntri_cell=None)
    with pytest.raises(_lib.GcError, match="no particles"):
        _create(empty)


def test_bad_topology_and_call_order(cuda_device):
    cfg = gen.small_channel()
    arrs = _cell_arrays(cfg)
    h = _create(cfg)
    try:
        def set_cells(a):
            _lib.call("gc_fused_set_cells", h, cfg.ncell, cfg.ntri, cfg.nedge, *[_ptr(x) for x in a])
        bad_tri = [x.copy() for x in arrs]
        bad_tri[0][0, 0] = cfg.ncp + 1
        with pytest.raises(_lib.GcError, match="triangle index"):
            set_cells(bad_tri)
        bad_edge = [x.copy() for x in arrs]
        bad_edge[1][3, 5] = cfg.ntri + 1
        with pytest.raises(_lib.GcError, match="edge triangle index"):
            set_cells(bad_edge)
        bad_range = [x.copy() for x in arrs]
        bad_range[2][0, 1] = cfg.ntri
        with pytest.raises(_lib.GcError, match="triangle range"):
            set_cells(bad_range)
        with pytest.raises(_lib.GcError, match="NULL array"):
            _lib.call("gc_fused_set_cells", h, cfg.ncell, cfg.ntri, cfg.nedge, *[_ptr(x) for x in arrs[:-1]],
                      C.c_void_p(0))
        set_cells(arrs)
        with pytest.raises(_lib.GcError, match="setup first"):
            _lib.call("gc_fused_step", h, 1, 1)
        with pytest.raises(_lib.GcError, match="setup first"):
            _lib.call("gc_fused_step_store", h, 1, *[C.c_void_p(0)] * 14)
        with pytest.raises(_lib.GcError, match="load the state"):
            _lib.call("gc_fused_setup", h)
        with pytest.raises(_lib.GcError, match="NULL"):
            _lib.call("gc_fused_load", h, C.c_void_p(0), C.c_void_p(0), C.c_void_p(0), C.c_void_p(0),
                      C.c_void_p(0), 0)
        pos = np.ascontiguousarray(cfg.coor, np.float32)
        vh = np.ascontiguousarray(cfg.velhalf, np.float32)
        _lib.call("gc_fused_load", h, _ptr(pos), C.c_void_p(0), _ptr(vh), C.c_void_p(0), C.c_void_p(0), 0)
        _lib.call("gc_fused_setup", h)
        with pytest.raises(_lib.GcError, match="already set up"):
            _lib.call("gc_fused_setup", h)
        with pytest.raises(_lib.GcError, match="before gc_fused_setup"):
            set_cells(arrs)
        with pytest.raises(_lib.GcError, match="nsteps"):
            _lib.call("gc_fused_step", h, -1, 1)
        with pytest.raises(_lib.GcError, match="outside"):
            _lib.call("gc_ensemble_diagnostics", h, 1, _ptr(np.zeros(8)))
        n = C.c_int()
        with pytest.raises(_lib.GcError, match="contact"):
            _lib.call("gc_ensemble_rouleaux", h, 0, C.c_float(-1.0), C.c_void_p(0), C.c_void_p(0), C.byref(n))
        _lib.call("gc_fused_step", h, 3, 1)   # the handle still works after the refusals
        _lib.call("gc_fused_step_store", h, 1, *[C.c_void_p(0)] * 14)   # a step, every output skipped
        flags = C.c_uint()
        _lib.call("gc_fused_flags", h, C.byref(flags))
        assert flags.value == 0
    finally:
        _destroy(h)
    fs = FusedSystem(cfg, noise=False)   # and so does the library
    fs.step(2, 1)
    assert fs.flags() == 0
    fs.close()
