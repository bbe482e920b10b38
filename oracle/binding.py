"""ctypes binding of the FP64 CPU oracle (oracle/oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke()
and by bench.py's CPU-baseline leg, never by the gpucell_gb300 package.
Parity against GPUCell itself is unpinned (its kernel bodies are not in the
reference); see oracle/oracle.c.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_HERE)
if _ROOT not in sys.path:
    sys.path.insert(0, _ROOT)

from gpucell_gb300._lib import Structconst  # noqa: E402  (the ABI struct, no compute)

LIB_PATH = os.path.join(_HERE, "build", "liboracle.so")

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)


class OrState(C.Structure):
    _fields_ = [
        ("c", Structconst), ("bbox", C.c_double * 6), ("pmask", C.c_int), ("noise_on", C.c_int),
        ("step", C.c_longlong), ("drive_on", C.c_int), ("nthreads", C.c_int),
        ("pos", _D), ("vel", _D), ("rho", _D), ("press", _D), ("force", _D), ("velhalf", _D), ("nthro", _I),
        ("ncell", C.c_int), ("ntri", C.c_int), ("nedge", C.c_int),
        ("tri", _I), ("edge", _I), ("betri", _I), ("celltab", _I),
        ("shearmod", _D), ("bendmod", _D), ("hlarea", _D), ("hgarea", _D), ("hvol", _D),
        ("refedgelen", _D), ("maxrefedgelen", _D), ("perlen", _D), ("hpow", _D), ("hbending", _D), ("refangle", _D),
        ("reftriarea", _D), ("refarea", _D), ("refvol", _D),
        ("triarea", _D), ("trinormal", _D), ("tricenter", _D), ("area", _D), ("vol", _D), ("pararea", _D),
        ("defforce", _D), ("aggforce", _D),
    ]


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from gpucell_gb300.build import build_oracle
            build_oracle()
        lib = C.CDLL(LIB_PATH)
        S = C.POINTER(OrState)
        for name in ("or_update_coor", "or_periodic", "or_density", "or_predict", "or_bound2_vel", "or_eos",
                     "or_sdpd_force", "or_rep_force", "or_ext_force", "or_mech_setup", "or_def_force",
                     "or_agg_force", "or_correct", "or_step"):
            getattr(lib, name).argtypes = [S]
            getattr(lib, name).restype = C.c_int
        lib.or_geo.argtypes = [S, C.c_int]
        lib.or_neighbor_stats.argtypes = [S, _I, C.POINTER(C.c_uint64)]
        lib.or_force_scale.argtypes = [S, C.c_int, _D]
        lib.or_force_scale.restype = C.c_int
        lib.or_membrane_energy.argtypes = [S]
        lib.or_membrane_energy.restype = C.c_double
        lib.or_morse_energy.argtypes = [S]
        lib.or_morse_energy.restype = C.c_double
        lib.or_pair_noise.argtypes = [S, C.c_uint, C.c_uint, _D]
        lib.or_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        lib.or_philox2x32_10.argtypes = [C.POINTER(C.c_uint32), C.c_uint32, C.POINTER(C.c_uint32)]
        lib.or_noise_key.argtypes = [C.c_uint64, C.c_uint64]
        lib.or_noise_key.restype = C.c_uint32
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(_D)


def _ip(a):
    return a.ctypes.data_as(_I)


class Oracle:
    """Oracle state for one configuration (arrays in original order)."""

    def __init__(self, cfg, noise=True, nthreads=0):
        self.lib = load()
        self.cfg = cfg
        n = cfg.n
        self.pos = cfg.coor.astype(np.float64).copy()
        self.vel = np.zeros((n, 3))
        self.rho = np.full(n, float(np.float32(cfg.den_init)))
        self.press = np.zeros(n)
        self.force = np.zeros((n, 3))
        self.velhalf = cfg.velhalf.astype(np.float64).copy()
        self.nthro = np.zeros((n, 3), np.int32)
        nt, ne, nc, ncp = cfg.ntri, cfg.nedge, cfg.ncell, cfg.ncp
        z = lambda *s: np.zeros(s if s else (1,))
        if nc:
            shear, bend, hl, hg, hv = cfg.edge_params()
            self.tri = np.ascontiguousarray(cfg.tri, np.int32)
            self.edge = np.ascontiguousarray(cfg.edge, np.int32)
            self.betri = np.ascontiguousarray(cfg.betri, np.int32)
            self.celltab = np.ascontiguousarray(cfg.celltab, np.int32)
            self.shearmod, self.bendmod = shear.astype(np.float64), bend.astype(np.float64)
            self.hlarea, self.hgarea, self.hvol = hl.astype(np.float64), hg.astype(np.float64), hv.astype(np.float64)
        else:
            self.tri = self.edge = self.betri = self.celltab = np.zeros(6, np.int32)
            self.shearmod = self.bendmod = self.hlarea = self.hgarea = self.hvol = z()
        for k, sz in (("refedgelen", ne), ("maxrefedgelen", ne), ("perlen", ne), ("hpow", ne), ("hbending", ne),
                      ("refangle", ne), ("reftriarea", nt), ("refarea", nc), ("refvol", nc), ("triarea", nt),
                      ("area", nc), ("vol", nc), ("pararea", ncp)):
            setattr(self, k, z(max(sz, 1)))
        self.trinormal, self.tricenter = z(max(nt, 1), 3), z(max(nt, 1), 3)
        self.defforce, self.aggforce = z(max(ncp, 1), 3), z(max(ncp, 1), 3)
        st = OrState()
        st.c = Structconst(**cfg.consts())
        for k in range(6):
            st.bbox[k] = float(cfg.bbox[k])
        st.pmask, st.noise_on, st.step, st.drive_on, st.nthreads = cfg.pmask, 1 if noise else 0, 0, 1, nthreads
        st.ncell, st.ntri, st.nedge = nc, nt, ne
        self.st = st
        self._bind()

    def _bind(self):
        st = self.st
        for k in ("pos", "vel", "rho", "press", "force", "velhalf", "shearmod", "bendmod", "hlarea", "hgarea", "hvol",
                  "refedgelen", "maxrefedgelen", "perlen", "hpow", "hbending", "refangle", "reftriarea", "refarea",
                  "refvol", "triarea", "trinormal", "tricenter", "area", "vol", "pararea", "defforce", "aggforce"):
            arr = getattr(self, k)
            assert arr.dtype == np.float64 and arr.flags.c_contiguous, k
            setattr(st, k, _dp(arr))
        for k in ("nthro", "tri", "edge", "betri", "celltab"):
            arr = getattr(self, k)
            assert arr.dtype == np.int32 and arr.flags.c_contiguous, k
            setattr(st, k, _ip(arr))

    def set(self, **arrays):
        """Copies arrays in (same names as the attributes)."""
        for k, v in arrays.items():
            cur = getattr(self, k)
            cur[...] = np.asarray(v, dtype=cur.dtype).reshape(cur.shape)

    def call(self, name, *args):
        rc = getattr(self.lib, "or_" + name)(C.byref(self.st), *args)
        if isinstance(rc, int) and rc != 0:
            raise RuntimeError(f"or_{name} failed ({rc})")
        return rc

    def neighbor_stats(self):
        n = self.cfg.n
        cnt = np.zeros(n, np.int32)
        h = np.zeros(n, np.uint64)
        self.lib.or_neighbor_stats(C.byref(self.st), _ip(cnt), h.ctypes.data_as(C.POINTER(C.c_uint64)))
        return cnt, h

    SCALE_SDPD, SCALE_REP, SCALE_BODY, SCALE_MEMB, SCALE_MORSE, SCALE_EOS, SCALE_ALL = 1, 2, 4, 8, 16, 32, 63

    def force_scale(self, parts=63):
        """Per particle, the sum of the magnitudes of the terms its force adds
        up (the parts selected by the SCALE_* bits), on the current state: the
        scale of FP32 rounding in the force."""
        out = np.zeros(self.cfg.n)
        rc = self.lib.or_force_scale(C.byref(self.st), int(parts), _dp(out))
        if rc != 0:
            raise RuntimeError(f"or_force_scale failed ({rc})")
        return out

    def forces_from_density(self, rho, press=None):
        """Re-evaluates every force of the current state in FP64 from the given
        densities and pressures (for instance a GPU's FP32 ones; without
        pressures, the EOS makes them): SDPD, wall repulsion, body force,
        membrane geometry and forces, aggregation.  Compared with the GPU's
        forces this isolates the force pass from the rounding of the density
        sum, which P = c^2 (rho - rho0) amplifies."""
        self.set(rho=rho)
        if press is None:
            self.call("eos")
        else:
            self.set(press=press)
        for name in ("sdpd_force", "rep_force", "ext_force"):
            self.call(name)
        if self.cfg.ncell:
            self.call("geo", 0)
            self.call("def_force")
            self.call("agg_force")

    def membrane_energy(self):
        return self.lib.or_membrane_energy(C.byref(self.st))

    def morse_energy(self):
        return self.lib.or_morse_energy(C.byref(self.st))

    def pair_noise(self, i, j):
        out = np.zeros(3)
        self.lib.or_pair_noise(C.byref(self.st), i, j, _dp(out))
        return out

    def setup(self):
        """CalGeoPara(StepCount -1) + SetMechPara (src/Particle.cu:476-480)."""
        if self.cfg.ncell:
            self.call("geo", 1)
            self.call("mech_setup")

    def step(self):
        return self.call("step")


def philox2(ctr, key):
    lib = load()
    c = (C.c_uint32 * 2)(*ctr)
    o = (C.c_uint32 * 2)()
    lib.or_philox2x32_10(c, key, o)
    return list(o)


def noise_key(seed, step):
    return int(load().or_noise_key(seed, step))


def philox(ctr, key):
    lib = load()
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib.or_philox4x32_10(c, k, o)
    return list(o)


# FP32 unit roundoff
U32 = 2.0 ** -24


def force_error_stats(got, want, scale, rtol=1e-5, k=16.0):
    """Per-particle comparison of forces (rows of 3) with the oracle's.

    Each particle i must satisfy |dF_i| <= rtol |F_i| + k u S_i, where u is
    FP32's unit roundoff and S_i the sum of the magnitudes of the terms F_i
    adds up (Oracle.force_scale): relative error rtol wherever the net force
    is not a cancellation of much larger terms, and a few roundings of the
    terms where it is.  Returns the median, 99th percentile and largest
    relative error |dF_i| / |F_i|, the fraction of particles within rtol
    relative, and the worst particle against the bound (ratio <= 1 passes)."""
    got = np.asarray(got, np.float64).reshape(-1, 3)
    want = np.asarray(want, np.float64).reshape(-1, 3)
    scale = np.asarray(scale, np.float64).reshape(-1)
    d = np.linalg.norm(got - want, axis=1)
    fn = np.linalg.norm(want, axis=1)
    ok = fn > 0
    rel = d[ok] / fn[ok]
    bound = rtol * fn + k * U32 * scale
    ratio = np.where(bound > 0, d / np.where(bound > 0, bound, 1.0), np.where(d > 0, np.inf, 0.0))
    w = int(np.argmax(ratio)) if ratio.size else -1
    return {
        "particles": int(d.size),
        "median_rel": float(np.median(rel)) if rel.size else 0.0,
        "p99_rel": float(np.percentile(rel, 99)) if rel.size else 0.0,
        "max_rel": float(rel.max()) if rel.size else 0.0,
        "frac_within_rtol": float((rel <= rtol).mean()) if rel.size else 1.0,
        "rtol": rtol, "k_roundoff": k,
        "worst_ratio": float(ratio[w]) if w >= 0 else 0.0,
        "worst": {"index": w, "dF": float(d[w]), "F": float(fn[w]), "scale": float(scale[w])} if w >= 0 else None,
    }


def assert_forces_close(got, want, scale, rtol=1e-5, k=16.0, what="force"):
    """force_error_stats, asserting that every particle is within its bound;
    the message names the worst particle."""
    s = force_error_stats(got, want, scale, rtol, k)
    assert s["worst_ratio"] <= 1.0, (
        f"{what}: particle {s['worst']['index']} has |dF| = {s['worst']['dF']:.3e} against |F| = "
        f"{s['worst']['F']:.3e} and term scale {s['worst']['scale']:.3e} (bound {rtol:g} |F| + {k:g} u S); "
        f"median rel {s['median_rel']:.2e}, p99 {s['p99_rel']:.2e}")
    return s
