"""GPUCell's input files through the library's loader (gc_input_*).

``read_inputs(directory)`` parses the four text files with the reference's
rules and no size caps; ``write_binary`` / ``read_binary`` keep the same set
in one binary file for fast reloading; ``to_config`` turns a set into the
``Config`` the rest of the package steps.
"""
from __future__ import annotations

import ctypes as C
import dataclasses

import numpy as np

from . import _lib
from .generator import Config, Physics, lattice_density  # noqa: F401

_ARRAYS = {
    # name: (count field or callable, columns, dtype)
    "sdpd_coor": (lambda s: s.n_b1 + s.n_b2 + s.n_fluid, 3, np.float32),
    "cell_type": ("ncell", 1, np.int32), "npar": ("ncell", 1, np.int32), "ntri_cell": ("ncell", 1, np.int32),
    "cell_coor": ("ncp", 3, np.float32), "tri": ("ntri", 3, np.int32), "edge": ("nedge", 6, np.int32),
    "betri": ("ncell", 2, np.int32), "celltab": ("ncp", 1, np.int32),
    "shear_mod": ("ntype", 1, np.float32), "bending_mod": ("ntype", 1, np.float32),
    "hgarea": ("ntype", 1, np.float32), "hlarea": ("ntype", 1, np.float32), "hvol": ("ntype", 1, np.float32),
    "shear_e": ("nedge", 1, np.float32), "bend_e": ("nedge", 1, np.float32), "hl_t": ("ntri", 1, np.float32),
    "hg_t": ("ntri", 1, np.float32), "hv_t": ("ntri", 1, np.float32),
}
_SCALARS = ("n_b1", "n_b2", "n_fluid", "sound1", "sound2", "shear_vis", "bulk_vis", "den_init", "ext_force",
            "ncell", "ntype", "ncp", "ntri", "nedge", "max_cut", "zero_len", "sca_fac", "sur_energy")


def _to_dict(s: _lib.GcInputSet) -> dict:
    out = {k: getattr(s, k) for k in _SCALARS}
    for name, (cnt, cols, dt) in _ARRAYS.items():
        n = cnt(s) if callable(cnt) else getattr(s, cnt)
        ptr = getattr(s, name)
        if not ptr or n == 0 or (name in ("shear_mod", "bending_mod", "hgarea", "hlarea", "hvol", "shear_e",
                                          "bend_e", "hl_t", "hg_t", "hv_t") and s.ncell == 0):
            a = np.zeros((n, cols) if cols > 1 else (n,), dt)
        else:
            a = np.ctypeslib.as_array(ptr, shape=(n * cols,)).astype(dt, copy=True)
            a = a.reshape(n, cols) if cols > 1 else a
        out[name] = a
    return out


def read_inputs(directory: str) -> dict:
    s = _lib.GcInputSet()
    _lib.call("gc_input_read", str(directory).encode(), C.byref(s))
    try:
        return _to_dict(s)
    finally:
        _lib.load().gc_input_free(C.byref(s))


def read_binary(path: str) -> dict:
    s = _lib.GcInputSet()
    _lib.call("gc_input_read_binary", str(path).encode(), C.byref(s))
    try:
        return _to_dict(s)
    finally:
        _lib.load().gc_input_free(C.byref(s))


def write_binary(directory_or_set, path: str) -> None:
    """Converts the four text files of a directory (or keeps a set already
    read) into one binary file."""
    s = _lib.GcInputSet()
    if isinstance(directory_or_set, str):
        _lib.call("gc_input_read", directory_or_set.encode(), C.byref(s))
        try:
            _lib.call("gc_input_write_binary", str(path).encode(), C.byref(s))
        finally:
            _lib.load().gc_input_free(C.byref(s))
        return
    d = directory_or_set
    keep = []
    for k in _SCALARS:
        setattr(s, k, d[k])
    for name, (_, _, dt) in _ARRAYS.items():
        a = np.ascontiguousarray(d[name], dt)
        keep.append(a)
        ctype = C.c_float if dt == np.float32 else C.c_int
        setattr(s, name, a.ctypes.data_as(C.POINTER(ctype)))
    _lib.call("gc_input_write_binary", str(path).encode(), C.byref(s))


def to_config(d: dict, phys: Physics | None = None, bbox=None, pmask: int = 1, name="inputs") -> Config:
    """A Config from an input set; constants the files do not carry (mass,
    time step, temperature, VVsigma, seed, cut-off) come from `phys`."""
    base = phys or Physics()
    p = dataclasses.replace(base, sound1=float(d["sound1"]), sound2=float(d["sound2"]),
                            shear_vis=float(d["shear_vis"]), bulk_vis=float(d["bulk_vis"]),
                            ext_force=float(d["ext_force"]), max_cut=float(d["max_cut"]),
                            zero_len=float(d["zero_len"]), sca_fac=float(d["sca_fac"]),
                            sur_energy=float(d["sur_energy"]))
    coor = np.concatenate([d["sdpd_coor"], d["cell_coor"]]).astype(np.float32)
    cfg = Config(name=name, bbox=np.asarray(bbox if bbox is not None else [0, 20, -10, 10, -10, 10], np.float32),
                 pmask=pmask, n_b1=int(d["n_b1"]), n_b2=int(d["n_b2"]), n_fluid=int(d["n_fluid"]), coor=coor,
                 velhalf=np.zeros_like(coor), den_init=float(d["den_init"]), phys=p)
    if d["ncell"]:
        cfg.ncell = int(d["ncell"])
        cfg.tri, cfg.edge, cfg.betri = d["tri"], d["edge"], d["betri"]
        cfg.celltab, cfg.npar, cfg.ntri_cell = d["celltab"], d["npar"], d["ntri_cell"]
        cfg.cell_type = d["cell_type"]
        cfg.moduli = (d["shear_e"], d["bend_e"], d["hl_t"], d["hg_t"], d["hv_t"])
    return cfg
