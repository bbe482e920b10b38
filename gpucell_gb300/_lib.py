"""ctypes binding of libgpucell_gb300.so (the C ABI in include/gpucell_gb300.h).

The library is the only compute path: if it is missing, importing the
binding raises instead of falling back to anything else.  Build it with
``python -c "import __graft_entry__ as g; g.build()"`` (or
``python -m gpucell_gb300.build``).
"""
from __future__ import annotations

import ctypes as C
import os

from .build import LIB_PATH

GC_OK = 0
GC_FLAG_NONFINITE = 1
GC_FLAG_BAD_INDEX = 2
GC_FLAG_CELL_OVERFLOW = 4
GC_FLAG_STRETCH = 8
GC_FLAG_TILE_FULL = 16


class Structconst(C.Structure):
    """ctypes mirror of Structconst (src/TypesDef.cuh:49-78), 96 bytes."""

    _fields_ = [
        ("nFluidStart", C.c_uint),
        ("nBound2Start", C.c_uint),
        ("nCellStart", C.c_uint),
        ("nTotalPar", C.c_uint),
        ("nCellPar", C.c_uint),
        ("iSeed", C.c_long),
        ("CutRadius", C.c_float),
        ("Mass", C.c_float),
        ("SoundSpeed1", C.c_float),
        ("SoundSpeed2", C.c_float),
        ("DenInit", C.c_float),
        ("VVsigma", C.c_float),
        ("ShearVis", C.c_float),
        ("BulkVis", C.c_float),
        ("ConstExtForce", C.c_float),
        ("TimeStep", C.c_float),
        ("surEnergy", C.c_float),
        ("MaxCut", C.c_float),
        ("zeroLen", C.c_float),
        ("scaFac", C.c_float),
        ("Temp", C.c_float),
    ]


assert C.sizeof(Structconst) == 96


class GcFusedOptions(C.Structure):
    """ctypes mirror of GcFusedOptions (include/gpucell_gb300.h)."""

    _fields_ = [("skin", C.c_float), ("block", C.c_int), ("list_capacity", C.c_int), ("compact", C.c_int),
                ("graph", C.c_int), ("tiles", C.c_int), ("fp32_positions", C.c_int),
                ("half_velocity", C.c_int)]


assert C.sizeof(GcFusedOptions) == 32


class GcSystemDesc(C.Structure):
    """ctypes mirror of GcSystemDesc (include/gpucell_gb300.h): one system of an ensemble."""

    _fields_ = [("consts", Structconst), ("bbox", C.c_float * 6), ("periodic_mask", C.c_int),
                ("reserved", C.c_int)]


assert C.sizeof(GcSystemDesc) == 128

GC_TUNE_CACHE = 1


class GcInputSet(C.Structure):
    """ctypes mirror of GcInputSet (include/gpucell_gb300.h)."""

    _FP = C.POINTER(C.c_float)
    _IP = C.POINTER(C.c_int)
    _fields_ = [("n_b1", C.c_longlong), ("n_b2", C.c_longlong), ("n_fluid", C.c_longlong), ("sdpd_coor", _FP),
                ("sound1", C.c_float), ("sound2", C.c_float), ("shear_vis", C.c_float), ("bulk_vis", C.c_float),
                ("den_init", C.c_float), ("ext_force", C.c_float), ("ncell", C.c_int), ("ntype", C.c_int),
                ("ncp", C.c_longlong), ("ntri", C.c_longlong), ("nedge", C.c_longlong), ("cell_type", _IP),
                ("npar", _IP), ("ntri_cell", _IP), ("cell_coor", _FP), ("tri", _IP), ("edge", _IP),
                ("betri", _IP), ("celltab", _IP), ("shear_mod", _FP), ("bending_mod", _FP), ("hgarea", _FP),
                ("hlarea", _FP), ("hvol", _FP), ("max_cut", C.c_float), ("zero_len", C.c_float),
                ("sca_fac", C.c_float), ("sur_energy", C.c_float), ("shear_e", _FP), ("bend_e", _FP),
                ("hl_t", _FP), ("hg_t", _FP), ("hv_t", _FP)]


class GcOutputFrame(C.Structure):
    """ctypes mirror of GcOutputFrame (include/gpucell_gb300.h)."""

    _fields_ = [("n", C.c_longlong), ("n_b1", C.c_longlong), ("n_b2", C.c_longlong), ("n_cell_start", C.c_longlong),
                ("pos", C.c_void_p), ("vel", C.c_void_p), ("rho", C.c_void_p), ("press", C.c_void_p),
                ("ncell", C.c_int), ("ntri", C.c_int), ("cell_verts", C.c_void_p), ("tri", C.c_void_p),
                ("betri", C.c_void_p), ("defforce", C.c_void_p), ("aggforce", C.c_void_p),
                ("tricenter", C.c_void_p), ("trinordir", C.c_void_p), ("cell_stats", C.c_void_p),
                ("threads", C.c_int), ("reserved", C.c_int)]

_P = C.c_void_p
_I = C.c_int
_U = C.c_uint
_L = C.c_long

# name -> argument types (all return int status unless listed in _RESTYPES)
_SIGS = {
    "gc_last_error": [],
    "gc_version": [],
    "gc_set_periodic": [_I],
    "gc_get_periodic": [],
    "gc_set_noise": [_I],
    "gc_set_engine": [_I],
    "gc_get_engine": [],
    "gc_set_step": [C.c_longlong],
    "gc_get_step": [],
    "gc_set_stream": [_P],
    "gc_device_status": [_P],
    "gc_scratch_bytes": [_P],
    "gc_shutdown": [],
    "gc_launch_count": [],
    "gc_cupar_ConstsDataUp": [_P],
    "gc_cupar_UpdateFluidCoor": [_I, _P, _P, _P, _P],
    "gc_cupar_AppFluidPeriodicBC": [_I, _P, _P, _P, _P],
    "gc_cupar_CalFluidDen": [_I, _P, _P, _P, _P, _P, _P, _P],
    "gc_cupar_PredictFluidVel": [_I, _P, _P, _P, _P],
    "gc_cupar_CalBound2Vel": [_I, _P, _P, _P, _P, _P, _P, _P],
    "gc_cupar_EOS": [_I, _P, _P, _P],
    "gc_cupar_CalFluidSDPDForce": [_I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P],
    "gc_cupar_CalFluidRepForce": [_I, _P, _P, _P, _P, _P, _P, _P],
    "gc_cupar_SetFluidExtForce": [_I, _I, _P, _P],
    "gc_cupar_CorrectFliudVel": [_I, _P, _P, _P, _P, _P, _P, _P, _P, _P],
    "gc_cupar_CalGeoPara": [_L, _I, _I] + [_P] * 17,
    "gc_cupar_SetMechPara": [_I, _I] + [_P] * 14,
    "gc_cupar_CalCellDefForce": [_I, _U, _U, _U, _U] + [_P] * 27,
    "gc_cupar_CalCellAggForce": [_U, _U, _U] + [_P] * 10,
    "gc_cudiv_PreConList": [_I, _I] + [_P] * 8,
    "gc_cudiv_Sort": [_I, _P, _P],
    "gc_cudiv_Sort_noalloc": [_I, _P, _P],
    "gc_cudiv_CalBeginEndCube": [_I, _I, _P, _P],
    "gc_cudiv_SortBasicArrays": [_I] + [_P] * 8,
    "gc_cudiv_SortArraysWithCells": [_I] + [_P] * 10,
    "gc_cudiv_Printf": [_I, _P, _P, _P],
    "gc_debug_neighbor_stats": [_I, _P, _P, _P, _P, _P],
    "gc_fused_create": [_P, _P, _I, _I, _P, _P],
    "gc_fused_set_cells": [_P, _I, _I, _I] + [_P] * 9,
    "gc_fused_load": [_P] * 6 + [_I],
    "gc_fused_setup": [_P],
    "gc_fused_step": [_P, _I, _I],
    "gc_fused_store": [_P] * 8 + [_I],
    "gc_fused_store_cells": [_P] * 8 + [_I],
    "gc_fused_step_store": [_P, _I] + [_P] * 14,
    "gc_fused_cell_sums": [_P, _P, _P],
    "gc_fused_stats": [_P] * 6,
    "gc_fused_flags": [_P, _P],
    "gc_fused_profile": [_P, _I],
    "gc_fused_profile_read": [_P, _P, _P, _P],
    "gc_fused_get_options": [_P, _P],
    "gc_fused_set_options": [_P, _P],
    "gc_fused_autotune": [_P, _I, _I, _I, _P, _P],
    "gc_fused_checkpoint": [_P, C.c_char_p],
    "gc_fused_restore": [_P, C.c_char_p],
    "gc_fused_destroy": [_P],
    "gc_ensemble_create": [_I, _P, _I, _P, _P],
    "gc_ensemble_size": [_P, _P, _P],
    "gc_ensemble_set_cells": [_P, _I, _I, _I, _I] + [_P] * 9,
    "gc_ensemble_load": [_P, _I] + [_P] * 5 + [_I],
    "gc_ensemble_store": [_P, _I] + [_P] * 7 + [_I],
    "gc_ensemble_store_cells": [_P, _I] + [_P] * 7 + [_I],
    "gc_ensemble_cell_sums": [_P, _I, _P, _P],
    "gc_ensemble_cell_stats": [_P, _I, _P],
    "gc_ensemble_diagnostics": [_P, _I, _P],
    "gc_ensemble_rouleaux": [_P, _I, C.c_float, _P, _P, _P],
    "gc_rouleaux_from_pairs": [_I, _I, _P, _P, _P, _P],
    "gc_ensemble_write_output": [_P, _I, C.c_char_p, C.c_longlong, C.c_double, _I, _I],
    "gc_fused_write_output": [_P, C.c_char_p, C.c_longlong, C.c_double, _I, _I],
    "gc_output_write": [_P, C.c_char_p, C.c_longlong, C.c_double, _I],
    "gc_input_read": [C.c_char_p, _P],
    "gc_input_write_binary": [C.c_char_p, _P],
    "gc_input_read_binary": [C.c_char_p, _P],
    "gc_input_free": [_P],
}
_RESTYPES = {"gc_last_error": C.c_char_p, "gc_get_step": C.c_longlong, "gc_launch_count": C.c_ulonglong}

_lib = None


class GcError(RuntimeError):
    """A gc_* call returned a non-zero status."""


def load(path: str | None = None):
    """Loads the library (once) and declares every exported signature."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: the CUDA library has not been built "
                           "(run `python -m gpucell_gb300.build`)")
    lib = C.CDLL(path)
    for name, args in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPES.get(name, C.c_int)
    _lib = lib
    return lib


def exported_symbols():
    return list(_SIGS)


def call(name: str, *args) -> int:
    """Calls gc_<name> and raises GcError on a non-zero status."""
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != GC_OK:
        msg = lib.gc_last_error().decode(errors="replace")
        raise GcError(f"{name} failed with status {rc}: {msg}")
    return rc


def launch_count() -> int:
    return int(load().gc_launch_count())


def device_status() -> int:
    lib = load()
    flags = C.c_uint(0)
    call("gc_device_status", C.byref(flags))
    return flags.value
