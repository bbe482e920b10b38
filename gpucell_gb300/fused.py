"""The fused timestep (gc_fused_* / gc_ensemble_* in include/gpucell_gb300.h)
from Python.

``FusedSystem`` loads a generated configuration in GPUCell's layouts into a
library-owned simulation, runs timesteps, and stores the state back in
original particle order, with host (numpy) or device (torch) buffers.
``Ensemble`` does the same for many independent configurations stepped by
the same launches.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _lib
from .generator import Config


def _ptr(a):
    if a is None:
        return C.c_void_p(0)
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(C.c_void_p)
    return C.c_void_p(a.data_ptr())


def _options(skin, block, list_capacity, compact, graph, tiles=False, fp32_positions=False, half_velocity=False):
    return _lib.GcFusedOptions(skin=skin, block=block, list_capacity=list_capacity, compact=1 if compact else 0,
                               graph=1 if graph else 0, tiles=1 if tiles else 0,
                               fp32_positions=1 if fp32_positions else 0, half_velocity=1 if half_velocity else 0)


def _cell_arrays(cfg: Config):
    shear, bend, hl, hg, hv = cfg.edge_params()
    return [np.ascontiguousarray(a) for a in (cfg.tri.astype(np.int32), cfg.edge.astype(np.int32),
                                              cfg.betri.astype(np.int32), cfg.celltab.astype(np.int32),
                                              shear, bend, hl, hg, hv)]


_PARTICLE_KEYS = ("pos", "vel", "rho", "press", "force", "velhalf", "nthro")
_CELL_KEYS = ("Area", "Vol", "DefForce", "AggForce", "TriNorDir", "TriCenter", "ParArea")


def _particle_out(n):
    return dict(pos=np.empty((n, 3), np.float32), vel=np.empty((n, 3), np.float32), rho=np.empty(n, np.float32),
                press=np.empty(n, np.float32), force=np.empty((n, 3), np.float32),
                velhalf=np.empty((n, 3), np.float32), nthro=np.empty((n, 3), np.int32))


def _cell_out(c: Config):
    return dict(Area=np.empty(c.ncell, np.float32), Vol=np.empty(c.ncell, np.float32),
                DefForce=np.empty((c.ncp, 3), np.float32), AggForce=np.empty((c.ncp, 3), np.float32),
                TriNorDir=np.empty((c.ntri, 3), np.float32), TriCenter=np.empty((c.ntri, 3), np.float32),
                ParArea=np.empty(c.ncp, np.float32))


class _Handle:
    """Calls shared by one simulation and an ensemble."""

    h: C.c_void_p

    def step(self, nsteps=1, drive_on=1):
        _lib.call("gc_fused_step", self.h, int(nsteps), int(drive_on))

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

    def options(self) -> dict:
        o = _lib.GcFusedOptions()
        _lib.call("gc_fused_get_options", self.h, C.byref(o))
        return dict(skin=round(float(o.skin), 6), block=o.block, list_capacity=o.list_capacity,
                    compact=bool(o.compact), graph=bool(o.graph), tiles=bool(o.tiles),
                    fp32_positions=bool(o.fp32_positions), half_velocity=bool(o.half_velocity))

    def set_options(self, skin=0.0, block=0, list_capacity=0, compact=None, graph=None, tiles=None):
        cur = self.options()
        o = _options(skin, block, list_capacity, cur["compact"] if compact is None else compact,
                     cur["graph"] if graph is None else graph, cur["tiles"] if tiles is None else tiles,
                     cur["fp32_positions"], cur["half_velocity"])
        _lib.call("gc_fused_set_options", self.h, C.byref(o))

    def autotune(self, trial_steps=30, drive_on=1, use_cache=False) -> dict:
        o = _lib.GcFusedOptions()
        ms = C.c_double()
        _lib.call("gc_fused_autotune", self.h, int(trial_steps), int(drive_on),
                  _lib.GC_TUNE_CACHE if use_cache else 0, C.byref(o), C.byref(ms))
        return dict(skin=round(float(o.skin), 6), block=o.block, compact=bool(o.compact), graph=bool(o.graph),
                    tiles=bool(o.tiles), ms_per_step=ms.value)

    def write_output(self, directory, step_data, time, first=False, sys=0, threads=0):
        """GPUCell's output files for one output step (see gpucell_gb300.output)."""
        _lib.call("gc_ensemble_write_output", self.h, int(sys), str(directory).encode(), int(step_data), float(time),
                  1 if first else 0, int(threads))

    def cell_stats(self, sys=0) -> np.ndarray:
        """Per-cell mean DefForce, mean AggForce, mean velocity (x, y, z each),
        |mean velocity|, area, volume: ncell x 12, reduced on the GPU in FP64."""
        cfg = self.cfgs[sys] if hasattr(self, "cfgs") else self.cfg
        out = np.zeros((max(cfg.ncell, 0), 12))
        if cfg.ncell:
            _lib.call("gc_ensemble_cell_stats", self.h, int(sys), _ptr(out))
        return out

    def diagnostics(self, sys=0) -> dict:
        """FP64 diagnostics reduced on the GPU: total momentum, kinetic energy,
        k_B T of the peculiar velocities, largest speed, mean fluid density,
        moving particles."""
        out = np.zeros(8)
        _lib.call("gc_ensemble_diagnostics", self.h, int(sys), _ptr(out))
        return dict(momentum=out[0:3].copy(), kinetic_energy=float(out[3]), temperature=float(out[4]),
                    max_speed=float(out[5]), mean_fluid_density=float(out[6]), moving=int(out[7]))

    def rouleaux(self, contact, sys=0) -> tuple[np.ndarray, np.ndarray]:
        """Rouleau label of every cell and the number of cells of each rouleau
        (cells in contact: a vertex pair closer than `contact`), found on the
        GPU (gc_ensemble_rouleaux)."""
        cfg = self.cfgs[sys] if hasattr(self, "cfgs") else self.cfg
        label = np.zeros(max(cfg.ncell, 1), np.int32)
        size = np.zeros(max(cfg.ncell, 1), np.int32)
        n = C.c_int()
        _lib.call("gc_ensemble_rouleaux", self.h, int(sys), float(contact), _ptr(label), _ptr(size), C.byref(n))
        return label[:cfg.ncell], size[:n.value]

    def checkpoint(self, path):
        _lib.call("gc_fused_checkpoint", self.h, str(path).encode())

    def restore(self, path):
        _lib.call("gc_fused_restore", self.h, str(path).encode())

    def close(self):
        if getattr(self, "h", None):
            _lib.call("gc_fused_destroy", self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class FusedSystem(_Handle):
    def __init__(self, cfg: Config, noise=True, skin=0.1, block=128, list_capacity=0, compact=True, graph=False,
                 tiles=False, fp32_positions=False, half_velocity=False):
        self.cfg = cfg
        self.lib = _lib.load()
        self.h = C.c_void_p()
        consts = _lib.Structconst(**cfg.consts())
        opt = _options(skin, block, list_capacity, compact, graph, tiles, fp32_positions, half_velocity)
        bbox = np.ascontiguousarray(cfg.bbox, np.float32)
        _lib.call("gc_fused_create", C.byref(consts), _ptr(bbox), cfg.pmask, 1 if noise else 0, C.byref(opt),
                  C.byref(self.h))
        if cfg.ncell:
            self._keep = _cell_arrays(cfg)
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

    def step_fetch(self, drive_on=1) -> dict:
        """One step and its outputs (gc_fused_step_store: what is final early
        in the step is copied while the step still runs); the keys of
        `fetch` but the FP64 cell sums."""
        out = _particle_out(self.cfg.n)
        c = self.cfg
        cells = _cell_out(c) if c.ncell else {k: None for k in _CELL_KEYS}
        _lib.call("gc_fused_step_store", self.h, int(drive_on), *[_ptr(out[k]) for k in _PARTICLE_KEYS],
                  *[_ptr(cells[k]) for k in _CELL_KEYS])
        if c.ncell:
            out.update(cells)
        return out

    def fetch(self) -> dict:
        out = _particle_out(self.cfg.n)
        _lib.call("gc_fused_store", self.h, *[_ptr(out[k]) for k in _PARTICLE_KEYS], 0)
        c = self.cfg
        if c.ncell:
            cells = _cell_out(c)
            _lib.call("gc_fused_store_cells", self.h, *[_ptr(cells[k]) for k in _CELL_KEYS], 0)
            out.update(cells)
            a, v = np.empty(c.ncell), np.empty(c.ncell)
            _lib.call("gc_fused_cell_sums", self.h, _ptr(a), _ptr(v))
            out["Area64"], out["Vol64"] = a, v
        return out


class Ensemble(_Handle):
    """Independent configurations of uneven size stepped by the same launches.

    The configurations must share their physical constants; particle counts,
    boxes, membranes, body force (``ConstExtForce``) and noise seed may
    differ.  ``fetch(s)`` gives system s in its own particle order, exactly as
    ``FusedSystem.fetch`` would.
    """

    def __init__(self, cfgs: Sequence[Config], noise=True, skin=0.1, block=128, list_capacity=0, compact=True,
                 graph=False, tiles=False):
        self.cfgs = list(cfgs)
        self.lib = _lib.load()
        self.h = C.c_void_p()
        descs = (_lib.GcSystemDesc * len(self.cfgs))()
        for d, cfg in zip(descs, self.cfgs):
            d.consts = _lib.Structconst(**cfg.consts())
            d.bbox[:] = [float(x) for x in cfg.bbox]
            d.periodic_mask = cfg.pmask
        opt = _options(skin, block, list_capacity, compact, graph, tiles)
        _lib.call("gc_ensemble_create", len(self.cfgs), descs, 1 if noise else 0, C.byref(opt), C.byref(self.h))
        self._keep = []
        for s, cfg in enumerate(self.cfgs):
            if cfg.ncell:
                arrs = _cell_arrays(cfg)
                self._keep.append(arrs)
                _lib.call("gc_ensemble_set_cells", self.h, s, cfg.ncell, cfg.ntri, cfg.nedge,
                          *[_ptr(a) for a in arrs])
            pos = np.ascontiguousarray(cfg.coor, np.float32)
            vh = np.ascontiguousarray(cfg.velhalf, np.float32)
            _lib.call("gc_ensemble_load", self.h, s, _ptr(pos), C.c_void_p(0), _ptr(vh), C.c_void_p(0),
                      C.c_void_p(0), 0)
        _lib.call("gc_fused_setup", self.h)

    @property
    def n(self) -> int:
        return sum(c.n for c in self.cfgs)

    def load(self, s, pos, vel=None, velhalf=None, force=None, nthro=None):
        arrs = [None if a is None else np.ascontiguousarray(a, np.int32 if k == 4 else np.float32)
                for k, a in enumerate((pos, vel, velhalf, force, nthro))]
        _lib.call("gc_ensemble_load", self.h, int(s), *[_ptr(a) for a in arrs], 0)

    def fetch(self, s) -> dict:
        c = self.cfgs[s]
        out = _particle_out(c.n)
        _lib.call("gc_ensemble_store", self.h, int(s), *[_ptr(out[k]) for k in _PARTICLE_KEYS], 0)
        if c.ncell:
            cells = _cell_out(c)
            _lib.call("gc_ensemble_store_cells", self.h, int(s), *[_ptr(cells[k]) for k in _CELL_KEYS], 0)
            out.update(cells)
            a, v = np.empty(c.ncell), np.empty(c.ncell)
            _lib.call("gc_ensemble_cell_sums", self.h, int(s), _ptr(a), _ptr(v))
            out["Area64"], out["Vol64"] = a, v
        return out
