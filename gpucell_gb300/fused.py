"""The fused timestep (gc_fused_* in include/gpucell_gb300.h) from Python.

``FusedSystem`` loads a generated configuration in GPUCell's layouts into a
library-owned simulation, runs timesteps, and stores the state back in
original particle order, with host (numpy) or device (torch) buffers.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .generator import Config


def _ptr(a):
    if a is None:
        return C.c_void_p(0)
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(C.c_void_p)
    return C.c_void_p(a.data_ptr())


class FusedSystem:
    def __init__(self, cfg: Config, noise=True, skin=0.1, block=128, list_capacity=0, compact=True):
        self.cfg = cfg
        self.lib = _lib.load()
        self.h = C.c_void_p()
        consts = _lib.Structconst(**cfg.consts())
        opt = _lib.GcFusedOptions(skin=skin, block=block, list_capacity=list_capacity, compact=1 if compact else 0)
        bbox = np.ascontiguousarray(cfg.bbox, np.float32)
        _lib.call("gc_fused_create", C.byref(consts), _ptr(bbox), cfg.pmask, 1 if noise else 0, C.byref(opt),
                  C.byref(self.h))
        if cfg.ncell:
            shear, bend, hl, hg, hv = cfg.edge_params()
            self._keep = [np.ascontiguousarray(a) for a in (cfg.tri.astype(np.int32), cfg.edge.astype(np.int32),
                                                           cfg.betri.astype(np.int32), cfg.celltab.astype(np.int32),
                                                           shear, bend, hl, hg, hv)]
            _lib.call("gc_fused_set_cells", self.h, cfg.ncell, cfg.ntri, cfg.nedge, *[_ptr(a) for a in self._keep])
        pos = np.ascontiguousarray(cfg.coor, np.float32)
        vh = np.ascontiguousarray(cfg.velhalf, np.float32)
        _lib.call("gc_fused_load", self.h, _ptr(pos), C.c_void_p(0), _ptr(vh), C.c_void_p(0), C.c_void_p(0), 0)
        _lib.call("gc_fused_setup", self.h)

    def load(self, pos, vel=None, velhalf=None, force=None, nthro=None):
        arrs = [None if a is None else np.ascontiguousarray(a, np.int32 if k == 4 else np.float32)
                for k, a in enumerate((pos, vel, velhalf, force, nthro))]
        _lib.call("gc_fused_load", self.h, *[_ptr(a) for a in arrs], 0)

    def setup(self):
        _lib.call("gc_fused_setup", self.h)

    def step(self, nsteps=1, drive_on=1):
        _lib.call("gc_fused_step", self.h, int(nsteps), int(drive_on))

    def fetch(self) -> dict:
        n = self.cfg.n
        out = dict(pos=np.empty((n, 3), np.float32), vel=np.empty((n, 3), np.float32), rho=np.empty(n, np.float32),
                   press=np.empty(n, np.float32), force=np.empty((n, 3), np.float32),
                   velhalf=np.empty((n, 3), np.float32), nthro=np.empty((n, 3), np.int32))
        _lib.call("gc_fused_store", self.h, *[_ptr(out[k]) for k in
                                             ("pos", "vel", "rho", "press", "force", "velhalf", "nthro")], 0)
        c = self.cfg
        if c.ncell:
            cells = dict(Area=np.empty(c.ncell, np.float32), Vol=np.empty(c.ncell, np.float32),
                         DefForce=np.empty((c.ncp, 3), np.float32), AggForce=np.empty((c.ncp, 3), np.float32),
                         TriNorDir=np.empty((c.ntri, 3), np.float32), TriCenter=np.empty((c.ntri, 3), np.float32),
                         ParArea=np.empty(c.ncp, np.float32))
            _lib.call("gc_fused_store_cells", self.h, *[_ptr(cells[k]) for k in
                                                       ("Area", "Vol", "DefForce", "AggForce", "TriNorDir",
                                                        "TriCenter", "ParArea")], 0)
            out.update(cells)
            a, v = np.empty(c.ncell), np.empty(c.ncell)
            _lib.call("gc_fused_cell_sums", self.h, _ptr(a), _ptr(v))
            out["Area64"], out["Vol64"] = a, v
        return out

    def stats(self) -> dict:
        r, s, cap, mx = C.c_longlong(), C.c_longlong(), C.c_int(), C.c_int()
        mean = C.c_double()
        _lib.call("gc_fused_stats", self.h, C.byref(r), C.byref(s), C.byref(cap), C.byref(mean), C.byref(mx))
        return dict(rebuilds=r.value, steps=s.value, capacity=cap.value, mean_neighbors=mean.value,
                    max_neighbors=mx.value)

    def flags(self) -> int:
        f = C.c_uint()
        _lib.call("gc_fused_flags", self.h, C.byref(f))
        return f.value

    def profile(self, enable=True):
        _lib.call("gc_fused_profile", self.h, 1 if enable else 0)

    def profile_read(self) -> dict:
        d, f, k = C.c_double(), C.c_double(), C.c_longlong()
        _lib.call("gc_fused_profile_read", self.h, C.byref(d), C.byref(f), C.byref(k))
        return dict(density_ms=d.value, force_ms=f.value, steps=k.value)

    def close(self):
        if self.h:
            _lib.call("gc_fused_destroy", self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
