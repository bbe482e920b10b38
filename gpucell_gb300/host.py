"""Host-side mirror of GPUCell's ``Particle`` class over the C ABI.

``ParticleSystem`` does what src/Particle.cu does around the GPU boundary:
it owns every device buffer in the reference layout (AllocGpuMemory,
src/Particle.cu:573-625), uploads the initial state (SetParticle and
ParticlesDataUp, :485-652), runs the set-up calls (ConstantDataUp,
ConCubeList, CalGeoPara with StepCount -1, SetMechPara; :471-483, :654-678)
and then one ``UpdatePar`` sequence per step (:1310-1329), calling the
library's extern "C" entry points in exactly the reference order.  Device
memory comes from PyTorch; all compute is in libgpucell_gb300.so.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .generator import Config


def reference_grid(bbox, rc=1.0):
    """nCube, OuterRegion, invWid and SizeCube exactly as
    Particle::ConfigDomain computes them (src/Particle.cu:551-560)."""
    b = [float(x) for x in bbox]
    ncube = [int(math.floor((b[1] - b[0]) / rc)), int(math.floor((b[3] - b[2] + 2.0 * rc) / rc)),
             int(math.floor((b[5] - b[4] + 2.0 * rc) / rc))]
    outer = [b[1] - b[0], b[3] - b[2] + 2.0 * rc, b[5] - b[4] + 2.0 * rc]
    invwid = [float(np.float32(ncube[k] / outer[k])) for k in range(3)]
    return ncube, outer, invwid, ncube[0] * ncube[1] * ncube[2]


class ParticleSystem:
    """One simulation on the GPU, driven through the reference-facing ABI."""

    def __init__(self, cfg: Config, device="cuda", noise=True):
        import torch

        self.torch = torch
        self.cfg = cfg
        self.dev = torch.device(device)
        self.lib = _lib.load()
        _lib.call("gc_set_periodic", cfg.pmask)
        _lib.call("gc_set_noise", 1 if noise else 0)
        n = cfg.n
        self.n = n
        self.ncube, self.outer, self.invwid, self.size_cube = reference_grid(cfg.bbox)
        f32, i32 = torch.float32, torch.int32
        z = lambda shape, dt=f32: torch.zeros(shape, dtype=dt, device=self.dev)
        d = {}
        d["TotalCoor"] = torch.as_tensor(cfg.coor, device=self.dev).contiguous()
        d["TotalForce"] = z((n, 3))
        d["nCube"] = torch.tensor(self.ncube, dtype=i32, device=self.dev)
        d["OuterRegion"] = torch.tensor(self.outer, dtype=f32, device=self.dev)
        d["invWid"] = torch.tensor(self.invwid, dtype=f32, device=self.dev)
        d["CC"] = z((n, 3), i32)
        d["CubePart"] = z(n, i32)
        d["SortPart"] = torch.arange(n, dtype=i32, device=self.dev)   # src/Particle.cu:562-565
        d["OldPos"] = z(n, i32)
        d["BeginEndCube"] = z((self.size_cube, 2), i32)
        vel = z((n, 4))
        vel[:, 3] = cfg.den_init                                       # src/Particle.cu:530
        d["Velrhop"] = vel
        d["VelHalf"] = torch.as_tensor(cfg.velhalf, device=self.dev).contiguous()
        d["Press"] = z(n)
        d["BBoxSDPD"] = torch.as_tensor(cfg.bbox, device=self.dev).contiguous()
        d["nThroBound"] = z((n, 3), i32)
        self.has_cells = cfg.ncell > 0
        if self.has_cells:
            ne, nt, nc, ncp = cfg.nedge, cfg.ntri, cfg.ncell, cfg.ncp
            shear, bend, hl, hg, hv = cfg.edge_params()
            T = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=self.dev)
            d["CellTab"] = T(cfg.celltab.astype(np.int32))
            d["CurPos"] = z(n, i32)
            d["Edge"] = T(cfg.edge.astype(np.int32))
            d["Tri"] = T(cfg.tri.astype(np.int32))
            d["BeginEndTri"] = T(cfg.betri.astype(np.int32))
            for k in ("TriNorDir", "TriCenter"):
                d[k] = z((nt, 3))
            for k in ("TriArea", "RefTriArea", "RefArea_Para", "RefVol_Para", "Area_Para", "Vol_Para"):
                d[k] = z(nt)
            for k in ("RefTriAngle", "RefEdgeLen", "PowerIndex", "PerLenWLC", "HPow", "HBending", "MaxRefEdgeLen"):
                d[k] = z(ne)
            d["ShearMod_Para"], d["BendingMod_Para"] = T(shear), T(bend)
            d["HLarea_Para"], d["HGarea_Para"], d["HVol_Para"] = T(hl), T(hg), T(hv)
            d["Area"], d["Vol"] = z(nc), z(nc)
            d["ParArea"] = z(ncp)
            d["DefForce"], d["AggForce"] = z((ncp, 3)), z((ncp, 3))
        self.d = d
        self.h_sdpdforce = np.zeros((n, 3), np.float32)   # host pointers the reference passes
        self.h_defforce = np.zeros((max(cfg.ncp, 1), 3), np.float32)
        self.consts = _lib.Structconst(**cfg.consts())
        self.step_count = -1                                # src/main.cu:23
        torch.cuda.synchronize(self.dev)
        self._setup()

    # -- pointers --------------------------------------------------------
    def p(self, name):
        return C.c_void_p(self.d[name].data_ptr()) if name in self.d else C.c_void_p(0)

    # -- src/Particle.cu:471-483 -----------------------------------------
    def _setup(self):
        _lib.call("gc_cupar_ConstsDataUp", C.byref(self.consts))     # :654-664
        self.con_cube_list()                                           # :570
        self.cal_geo_para()                                            # :476 (StepCount -1)
        if self.has_cells:
            p = self.p
            _lib.call("gc_cupar_SetMechPara", self.cfg.ncell, self.cfg.nedge, p("Edge"), p("CurPos"), p("RefEdgeLen"),
                      p("MaxRefEdgeLen"), p("BendingMod_Para"), p("ShearMod_Para"), p("HBending"), p("PowerIndex"),
                      p("PerLenWLC"), p("HPow"), p("RefTriAngle"), p("TriNorDir"), p("TriCenter"), p("TotalCoor"))
        self.step_count += 1

    def con_cube_list(self):   # src/Particle.cu:666-678
        p, n = self.p, self.n
        _lib.call("gc_cudiv_PreConList", n, 1, p("TotalCoor"), p("BBoxSDPD"), p("invWid"), p("nCube"), p("CC"),
                  p("CubePart"), p("SortPart"), p("OldPos"))
        _lib.call("gc_cudiv_Sort", n, p("CubePart"), p("SortPart"))
        _lib.call("gc_cudiv_CalBeginEndCube", n, self.size_cube, p("CubePart"), p("BeginEndCube"))
        if self.has_cells:
            _lib.call("gc_cudiv_SortArraysWithCells", n, p("SortPart"), p("OldPos"), p("CurPos"), p("TotalCoor"),
                      p("CC"), p("Velrhop"), p("VelHalf"), p("TotalForce"), p("Press"), p("nThroBound"))
        else:
            _lib.call("gc_cudiv_SortBasicArrays", n, p("SortPart"), p("OldPos"), p("TotalCoor"), p("CC"),
                      p("Velrhop"), p("VelHalf"), p("TotalForce"), p("Press"))

    def cal_geo_para(self):   # src/Particle.cu:476, :1322
        if not self.has_cells:
            return
        p = self.p
        _lib.call("gc_cupar_CalGeoPara", self.step_count, self.cfg.ntri, self.cfg.ncell, p("BBoxSDPD"), p("CurPos"),
                  p("Tri"), p("BeginEndTri"), p("nThroBound"), p("TotalCoor"), p("TriNorDir"), p("TriArea"),
                  p("RefTriArea"), p("TriCenter"), p("RefArea_Para"), p("RefVol_Para"), p("Area_Para"),
                  p("Vol_Para"), p("Area"), p("Vol"), p("ParArea"))

    # -- individual stages of UpdatePar (src/Particle.cu:1331-1391) -------
    def update_coor(self):
        p = self.p
        _lib.call("gc_cupar_UpdateFluidCoor", self.n, p("SortPart"), p("TotalForce"), p("TotalCoor"), p("Velrhop"))

    def periodic(self):
        p = self.p
        _lib.call("gc_cupar_AppFluidPeriodicBC", self.n, p("SortPart"), p("TotalCoor"), p("nThroBound"),
                  p("BBoxSDPD"))

    def density(self):
        p = self.p
        _lib.call("gc_cupar_CalFluidDen", self.n, p("TotalCoor"), p("Velrhop"), p("CC"), p("nCube"),
                  p("OuterRegion"), p("SortPart"), p("BeginEndCube"))

    def predict(self):
        p = self.p
        _lib.call("gc_cupar_PredictFluidVel", self.n, p("SortPart"), p("Velrhop"), p("VelHalf"), p("TotalForce"))

    def bound2_vel(self):
        p = self.p
        _lib.call("gc_cupar_CalBound2Vel", self.n, p("TotalCoor"), p("Velrhop"), p("CC"), p("nCube"),
                  p("OuterRegion"), p("SortPart"), p("BeginEndCube"))

    def eos(self):
        p = self.p
        _lib.call("gc_cupar_EOS", self.n, p("SortPart"), p("Velrhop"), p("Press"))

    def sdpd_force(self):
        p = self.p
        _lib.call("gc_cupar_CalFluidSDPDForce", self.n, self.h_sdpdforce.ctypes.data_as(C.c_void_p), p("TotalCoor"),
                  p("Velrhop"), p("CC"), p("nCube"), p("SortPart"), p("OuterRegion"), p("BeginEndCube"),
                  p("TotalForce"), p("Press"))

    def rep_force(self):
        p = self.p
        _lib.call("gc_cupar_CalFluidRepForce", self.n, p("TotalCoor"), p("CC"), p("nCube"), p("SortPart"),
                  p("OuterRegion"), p("BeginEndCube"), p("TotalForce"))

    def ext_force(self, drive_on=1):
        p = self.p
        _lib.call("gc_cupar_SetFluidExtForce", int(drive_on), self.n, p("SortPart"), p("TotalForce"))

    def def_force(self):
        if not self.has_cells:
            return
        p, c = self.p, self.cfg
        _lib.call("gc_cupar_CalCellDefForce", c.ncell, c.nedge, c.ntri, self.n, c.ncp, p("BBoxSDPD"), p("Edge"),
                  p("Tri"), p("TotalCoor"), self.h_defforce.ctypes.data_as(C.c_void_p), p("DefForce"),
                  p("nThroBound"), p("MaxRefEdgeLen"), p("PowerIndex"), p("PerLenWLC"), p("HPow"), p("TriNorDir"),
                  p("TriCenter"), p("RefTriAngle"), p("HBending"), p("TriArea"), p("RefTriArea"), p("HLarea_Para"),
                  p("HGarea_Para"), p("Area_Para"), p("RefArea_Para"), p("HVol_Para"), p("Vol_Para"),
                  p("RefVol_Para"), p("TotalForce"), p("SortPart"), p("CurPos"))

    def agg_force(self):
        if not self.has_cells:
            return
        p, c = self.p, self.cfg
        _lib.call("gc_cupar_CalCellAggForce", c.ncell, self.n, c.ncp, p("TotalCoor"), p("AggForce"), p("CC"),
                  p("nCube"), p("SortPart"), p("CellTab"), p("OuterRegion"), p("BeginEndCube"), p("TotalForce"),
                  p("ParArea"))

    def correct(self):
        p = self.p
        _lib.call("gc_cupar_CorrectFliudVel", self.n, p("SortPart"), p("TotalForce"), p("VelHalf"), p("Velrhop"),
                  p("TotalCoor"), p("CC"), p("nCube"), p("OuterRegion"), p("BeginEndCube"))

    def update(self, drive_on=None):
        """One step: Particle::DrivePar + UpdatePar (src/Particle.cu:1302-1329)."""
        if drive_on is None:
            drive_on = 1 if self.step_count >= 0 else 0
        self.update_coor()
        self.periodic()
        self.con_cube_list()
        self.density()
        self.predict()
        self.bound2_vel()
        self.eos()
        self.sdpd_force()
        self.rep_force()
        self.ext_force(drive_on)
        self.cal_geo_para()
        self.def_force()
        self.agg_force()
        self.correct()
        self.bound2_vel()
        self.step_count += 1

    # -- host views --------------------------------------------------------
    def sortpart(self) -> np.ndarray:
        return self.d["SortPart"].cpu().numpy()

    def fetch(self) -> dict:
        """ParticlesDataReturn (src/Particle.cu:693-710), reordered to
        original ids.  Membrane arrays are already in original order."""
        sp = self.sortpart()
        inv = np.empty_like(sp)
        inv[sp] = np.arange(sp.size, dtype=sp.dtype)
        g = lambda k: self.d[k].cpu().numpy()[inv]
        vr = g("Velrhop")
        out = dict(pos=g("TotalCoor"), vel=vr[:, :3], rho=vr[:, 3], press=g("Press"), force=g("TotalForce"),
                   velhalf=g("VelHalf"), nthro=g("nThroBound"), cc=g("CC"), slot_of=inv, sortpart=sp)
        if self.has_cells:
            for k in ("Area", "Vol", "DefForce", "AggForce", "ParArea", "TriNorDir", "TriCenter", "TriArea",
                      "RefTriArea", "RefArea_Para", "RefVol_Para", "Area_Para", "Vol_Para", "RefEdgeLen",
                      "MaxRefEdgeLen", "PerLenWLC", "HPow", "HBending", "RefTriAngle", "PowerIndex"):
                out[k] = self.d[k].cpu().numpy()
        return out

    def set_state(self, **arrays):
        """Scatters original-order host arrays into slot order: pos, vel,
        rho, press, force, velhalf, nthro."""
        torch = self.torch
        sp = torch.as_tensor(self.sortpart().astype(np.int64), device=self.dev)
        m = {"pos": ("TotalCoor", None), "vel": ("Velrhop", slice(0, 3)), "rho": ("Velrhop", 3),
             "press": ("Press", None), "force": ("TotalForce", None), "velhalf": ("VelHalf", None),
             "nthro": ("nThroBound", None)}
        for k, v in arrays.items():
            name, sl = m[k]
            t = torch.as_tensor(np.asarray(v), device=self.dev).to(self.d[name].dtype)
            if sl is None:
                self.d[name][:] = t[sp]
            else:
                self.d[name][:, sl] = t[sp]
        torch.cuda.synchronize(self.dev)
