"""GPUCell's output files (OutputPar, src/Particle.cu:681-1300) from Python.

``write_frame`` hands host arrays to the library's writer
(``gc_output_write``); ``FusedSystem.write_output`` / ``Ensemble.write_output``
store a simulation and write it in one call.  ``read_plt`` reads any of the
files back into zones of float rows (for checks and post-processing).
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional

import numpy as np

from . import _lib


def _p(a):
    return C.c_void_p(0) if a is None else a.ctypes.data_as(C.c_void_p)


def write_frame(directory: str, step_data: int, time: float, first: bool, *, pos, vel, rho, press, n_b1: int,
                n_b2: int, n_cell_start: int, cell_verts=None, tri=None, betri=None, defforce=None, aggforce=None,
                tricenter=None, trinordir=None, cell_stats=None, threads: int = 0) -> None:
    """Writes one output step from host arrays in original particle order
    (membrane arrays in membrane order, `tri` 1-based, `cell_verts` and
    `betri` as inclusive ranges, `cell_stats` ncell x 12)."""
    f32 = lambda a: None if a is None else np.ascontiguousarray(a, np.float32)
    i32 = lambda a: None if a is None else np.ascontiguousarray(a, np.int32)
    keep = dict(pos=f32(pos), vel=f32(vel), rho=f32(rho), press=f32(press), cell_verts=i32(cell_verts),
                tri=i32(tri), betri=i32(betri), defforce=f32(defforce), aggforce=f32(aggforce),
                tricenter=f32(tricenter), trinordir=f32(trinordir),
                cell_stats=None if cell_stats is None else np.ascontiguousarray(cell_stats, np.float64))
    n = keep["pos"].shape[0]
    fr = _lib.GcOutputFrame()
    fr.n, fr.n_b1, fr.n_b2, fr.n_cell_start = n, n_b1, n_b2, n_cell_start
    for k in ("pos", "vel", "rho", "press", "cell_verts", "tri", "betri", "defforce", "aggforce", "tricenter",
              "trinordir", "cell_stats"):
        setattr(fr, k, _p(keep[k]))
    fr.ncell = 0 if keep["betri"] is None else keep["betri"].reshape(-1, 2).shape[0]
    fr.ntri = 0 if keep["tri"] is None else keep["tri"].reshape(-1, 3).shape[0]
    fr.threads = threads
    _lib.call("gc_output_write", C.byref(fr), directory.encode(), int(step_data), float(time), 1 if first else 0)


def read_plt(path: str) -> List[dict]:
    """Zones of a Tecplot file written in the reference's format: each zone
    is {"header": the zone line (or None before the first), "rows": float
    array}.  Rows with a different number of columns (the triangle
    connectivity of FE zones) go to "conn"."""
    zones: List[dict] = []
    cur: Optional[dict] = None
    with open(path) as f:
        for line in f:
            s = line.strip()
            if not s or s.startswith("Title=") or s.startswith("Variables="):
                continue
            if s.startswith("Zone"):
                cur = {"header": s, "rows": [], "conn": []}
                zones.append(cur)
                continue
            if cur is None:
                cur = {"header": None, "rows": [], "conn": []}
                zones.append(cur)
            vals = s.split()
            if cur["rows"] and len(vals) != len(cur["rows"][0]):
                cur["conn"].append([int(v) for v in vals])
            else:
                cur["rows"].append([float(v) for v in vals])
    for z in zones:
        z["rows"] = np.asarray(z["rows"], np.float64)
        z["conn"] = np.asarray(z["conn"], np.int64)
    return zones
