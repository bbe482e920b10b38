"""Seeded synthetic inputs in GPUCell's layout.

GPUCell reads four fixed-width text files (src/Particle.cu:45-427); no
input set ships with the reference, so the workloads are generated here:

* particles in original-id order: Bound1 walls, Bound2 walls, fluid,
  membrane vertices (src/Particle.cu:432-435);
* membranes as icosphere meshes mapped onto the Evans & Fung (1972)
  biconcave red-cell shape, with triangles ``(v1, v2, v3)`` and edge records
  ``(p1, p2, p3, p4, t1, t2)`` using the reference's 1-based, per-cell-offset
  indexing (src/Particle.cu:174-303);
* per-type membrane moduli broadcast to edges and triangles as
  src/Particle.cu:405-425 does.

Lengths are in units of the cut-off radius (CutRadius = 1, as
src/main.cuh:11 requires), with lattice spacing dx = rc/3 (Wendland C2 with
h = 1.5 dx).  ``write_reference_inputs`` writes the four text files, and
``read_reference_inputs`` parses them back with the reference's column rules.
"""
from __future__ import annotations

import dataclasses
import math
import os
from typing import Optional

import numpy as np

# Evans & Fung (1972) red-cell profile: half-thickness
#   z(s) = D0 sqrt(1 - s^2) (a0 + a1 s^2/4 + a2 s^4/16),  s = 2 r / D0
EF_A0, EF_A1, EF_A2 = 0.0518, 2.0026, -4.491


@dataclasses.dataclass
class Physics:
    """Reduced-unit parameters (rc = 1, m = 1)."""

    sound1: float = 20.0       # SoundSpeed1 (fluid, Bound2)
    sound2: float = 20.0       # SoundSpeed2 (membrane)
    shear_vis: float = 10.0    # eta
    bulk_vis: float = 0.0      # zeta
    ext_force: float = 0.02    # ConstExtForce / Mass
    temp: float = 1.0          # kT
    dt: float = 1.0e-3         # TimeStep (src/main.cuh:8)
    mass: float = 1.0
    vvsigma: float = 0.65      # src/Particle.cu:436
    seed: int = 1              # iSeed (src/Particle.cu:437)
    # membrane (one cell type)
    shear_mod: float = 100.0
    bending_mod: float = 50.0
    hgarea: float = 5000.0
    hlarea: float = 100.0
    hvol: float = 5000.0
    # Morse aggregation (0 = off)
    sur_energy: float = 0.0
    max_cut: float = 0.0
    zero_len: float = 0.0
    sca_fac: float = 0.0


@dataclasses.dataclass
class Config:
    name: str
    bbox: np.ndarray                 # (6,) float32: lo_x hi_x lo_y hi_y lo_z hi_z
    pmask: int                       # periodic axes
    n_b1: int
    n_b2: int
    n_fluid: int
    coor: np.ndarray                 # (N, 3) float32, original order
    velhalf: np.ndarray              # (N, 3) float32 (prescribed wall velocity for Bound2)
    den_init: float
    phys: Physics
    # membranes
    ncell: int = 0
    npar: Optional[np.ndarray] = None      # (ncell,) vertices per cell
    ntri_cell: Optional[np.ndarray] = None
    tri: Optional[np.ndarray] = None       # (ntri, 3) int32, 1-based membrane index
    edge: Optional[np.ndarray] = None      # (nedge, 6) int32
    betri: Optional[np.ndarray] = None     # (ncell, 2) int32
    celltab: Optional[np.ndarray] = None   # (ncp,) int32
    cell_type: Optional[np.ndarray] = None # (ncell,) 1-based
    meta: dict = dataclasses.field(default_factory=dict)   # how the configuration was drawn
    moduli: Optional[tuple] = None         # per-edge shear, bending; per-triangle hl, hg, hv (else from phys)

    @property
    def n(self) -> int:
        return int(self.coor.shape[0])

    @property
    def ncp(self) -> int:
        return 0 if self.celltab is None else int(self.celltab.shape[0])

    @property
    def ntri(self) -> int:
        return 0 if self.tri is None else int(self.tri.shape[0])

    @property
    def nedge(self) -> int:
        return 0 if self.edge is None else int(self.edge.shape[0])

    @property
    def n_cell_start(self) -> int:
        return self.n_b1 + self.n_b2 + self.n_fluid

    def consts(self) -> dict:
        """Fields of Structconst as the host frame fills them
        (src/Particle.cu:124-172, :429-437, :654-660)."""
        p = self.phys
        return dict(
            nBound2Start=self.n_b1,
            nFluidStart=self.n_b1 + self.n_b2,
            nCellStart=self.n_cell_start,
            nTotalPar=self.n,
            nCellPar=self.ncp,
            iSeed=p.seed,
            CutRadius=1.0,
            Mass=p.mass,
            SoundSpeed1=p.sound1,
            SoundSpeed2=p.sound2,
            DenInit=self.den_init,
            VVsigma=p.vvsigma,
            ShearVis=p.shear_vis,
            BulkVis=p.bulk_vis,
            ConstExtForce=p.ext_force * p.mass,
            TimeStep=p.dt,
            surEnergy=p.sur_energy,
            MaxCut=p.max_cut,
            zeroLen=p.zero_len,
            scaFac=p.sca_fac,
            Temp=p.temp,
        )

    def edge_params(self):
        """Per-edge shear and bending moduli, per-triangle area/volume constants."""
        if self.moduli is not None:
            return tuple(np.ascontiguousarray(a, np.float32) for a in self.moduli)
        p = self.phys
        return (np.full(self.nedge, p.shear_mod, np.float32), np.full(self.nedge, p.bending_mod, np.float32),
                np.full(self.ntri, p.hlarea, np.float32), np.full(self.ntri, p.hgarea, np.float32),
                np.full(self.ntri, p.hvol, np.float32))


# ---------------------------------------------------------------------------
# meshes
# ---------------------------------------------------------------------------

def icosphere(subdiv: int):
    """Unit icosphere: (V, 3) float64 vertices, (F, 3) int32 outward triangles."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], float)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(subdiv):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        key = np.sort(e, axis=1)
        uniq, inv = np.unique(key, axis=0, return_inverse=True)
        mid = v[uniq[:, 0]] + v[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        nv = v.shape[0]
        m = inv.reshape(3, -1) + nv   # midpoint of (0,1), (1,2), (2,0) per face
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        mab, mbc, mca = m[0], m[1], m[2]
        f = np.concatenate([np.stack([a, mab, mca], 1), np.stack([b, mbc, mab], 1), np.stack([c, mca, mbc], 1),
                            np.stack([mab, mbc, mca], 1)])
        v = np.concatenate([v, mid])
    # make every face outward
    cen = v[f].mean(axis=1)
    nrm = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    flip = (nrm * cen).sum(1) < 0
    f[flip] = f[flip][:, [0, 2, 1]]
    return v, f.astype(np.int32)


def biconcave(v_unit: np.ndarray, diameter: float) -> np.ndarray:
    """Maps unit-sphere vertices onto the Evans-Fung red-cell shape of the
    given diameter, axis along z."""
    x, y, z = v_unit[:, 0], v_unit[:, 1], v_unit[:, 2]
    s2 = x * x + y * y
    prof = EF_A0 + EF_A1 * s2 / 4.0 + EF_A2 * s2 * s2 / 16.0
    return np.stack([0.5 * diameter * x, 0.5 * diameter * y, diameter * z * prof], axis=1)


def edge_records(faces: np.ndarray) -> np.ndarray:
    """(p1, p2, p3, p4, t1, t2) per undirected edge, 0-based: p1-p2 is the
    shared edge, p3 the opposite vertex in t1 (where the edge runs p1 -> p2)
    and p4 the opposite vertex in t2."""
    F = faces.shape[0]
    tid = np.arange(F)
    u = np.concatenate([faces[:, 0], faces[:, 1], faces[:, 2]])
    w = np.concatenate([faces[:, 1], faces[:, 2], faces[:, 0]])
    opp = np.concatenate([faces[:, 2], faces[:, 0], faces[:, 1]])
    t = np.concatenate([tid, tid, tid])
    fwd = u < w
    key = np.minimum(u, w).astype(np.int64) * (faces.max() + 1) + np.maximum(u, w)
    kf, kb = key[fwd], key[~fwd]
    of, ob = np.argsort(kf), np.argsort(kb)
    if kf.shape != kb.shape or not np.array_equal(kf[of], kb[ob]):
        raise ValueError("mesh is not a closed, consistently oriented surface")
    uf, wf, pf, tf = u[fwd][of], w[fwd][of], opp[fwd][of], t[fwd][of]
    pb, tb = opp[~fwd][ob], t[~fwd][ob]
    return np.stack([uf, wf, pf, pb, tf, tb], axis=1).astype(np.int32)


def random_rotation(rng) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                     [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                     [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def lattice_density(dx: float, rc: float = 1.0) -> float:
    """Wendland C2 kernel sum (including self) on a simple-cubic lattice."""
    k = int(math.ceil(rc / dx)) + 1
    g = np.arange(-k, k + 1) * dx
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    r = np.sqrt(X * X + Y * Y + Z * Z)
    s = r[r < rc] / rc
    return float((21.0 / (2.0 * math.pi * rc ** 3) * (1 - s) ** 4 * (1 + 4 * s)).sum())


# ---------------------------------------------------------------------------
# assembly
# ---------------------------------------------------------------------------

def _assemble(name, bbox, pmask, b1, b2, fluid, cells, phys, dx, wall_vel=None) -> Config:
    """cells: list of (vertices (V,3), faces (F,3) 0-based)."""
    parts = [np.asarray(a, np.float32).reshape(-1, 3) for a in (b1, b2, fluid)]
    n_b1, n_b2, n_fl = (p.shape[0] for p in parts)
    coor = np.concatenate(parts + [np.asarray(c[0], np.float32) for c in cells]) if cells else np.concatenate(parts)
    velhalf = np.zeros_like(coor)
    if wall_vel is not None:
        velhalf[n_b1:n_b1 + n_b2] = wall_vel
    cfg = Config(name=name, bbox=np.asarray(bbox, np.float32), pmask=pmask, n_b1=n_b1, n_b2=n_b2, n_fluid=n_fl,
                 coor=coor, velhalf=velhalf, den_init=phys.mass * lattice_density(dx), phys=phys)
    if cells:
        tris, edges, betri, celltab, npar, ntri = [], [], [], [], [], []
        voff = toff = 0
        for c, (verts, faces) in enumerate(cells):
            nv, nf = verts.shape[0], faces.shape[0]
            er = edge_records(faces)
            tris.append(faces + 1 + voff)                    # 1-based + vertex offset b
            e = er.copy()
            e[:, :4] += 1 + voff                             # vertices: 1-based + b
            e[:, 4:] += 1 + toff                             # triangles: 1-based + a
            edges.append(e)
            betri.append([toff, toff + nf - 1])
            celltab.append(np.full(nv, c, np.int32))
            npar.append(nv)
            ntri.append(nf)
            voff += nv
            toff += nf
        cfg.ncell = len(cells)
        cfg.tri = np.concatenate(tris).astype(np.int32)
        cfg.edge = np.concatenate(edges).astype(np.int32)
        cfg.betri = np.asarray(betri, np.int32)
        cfg.celltab = np.concatenate(celltab)
        cfg.npar = np.asarray(npar, np.int32)
        cfg.ntri_cell = np.asarray(ntri, np.int32)
        cfg.cell_type = np.ones(len(cells), np.int32)
    return cfg


def _lattice(nx, ny, nz, dx, origin, rng, jitter=0.05):
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    p = np.stack([i.ravel(), j.ravel(), k.ravel()], 1).astype(np.float64)
    p = (p + 0.5) * dx + np.asarray(origin, float)
    if jitter:
        p += rng.uniform(-jitter * dx, jitter * dx, size=p.shape)
    return p


def channel(nx=64, ny=32, nz=32, wall_layers=3, b1_layers=0, cell_subdiv=3, cell_diameter=None, seed=12345,
            phys: Physics | None = None, wall_vel=None, name="channel", cell_centers=None) -> Config:
    """Poiseuille channel: fluid lattice nx*ny*nz (dx = 1/3), walls of
    `wall_layers` Bound2 layers in y on both sides (plus `b1_layers` Bound1
    layers outside them), periodic in x and z, one red cell in the middle
    (cell_subdiv < 0: none; `cell_centers` places one cell at each offset
    from the middle instead).  The default is the 65,536-fluid channel with
    3 wall layers and one 642-vertex cell of 8 um at dx = 0.5 um."""
    phys = phys or Physics()
    rng = np.random.default_rng(seed)
    dx = 1.0 / 3.0
    Lx, Ly, Lz = nx * dx, ny * dx, nz * dx
    bbox = [0.0, Lx, -Ly / 2, Ly / 2, -Lz / 2, Lz / 2]
    fluid = _lattice(nx, ny, nz, dx, (0.0, -Ly / 2, -Lz / 2), rng)
    xs = (np.arange(nx) + 0.5) * dx
    zs = (np.arange(nz) + 0.5) * dx - Lz / 2
    X, Z = np.meshgrid(xs, zs, indexing="ij")

    def layer(y):
        return np.stack([X.ravel(), np.full(X.size, y), Z.ravel()], 1)

    b2 = [layer(-Ly / 2 - (k + 0.5) * dx) for k in range(wall_layers)] + \
         [layer(Ly / 2 + (k + 0.5) * dx) for k in range(wall_layers)]
    b1 = [layer(-Ly / 2 - (wall_layers + k + 0.5) * dx) for k in range(b1_layers)] + \
         [layer(Ly / 2 + (wall_layers + k + 0.5) * dx) for k in range(b1_layers)]
    cells = []
    if cell_subdiv >= 0:
        d = cell_diameter if cell_diameter is not None else 8.0 / 1.5   # 8 um at rc = 3 dx = 1.5 um
        v, f = icosphere(cell_subdiv)
        shape = biconcave(v, d)
        rot = np.array([[1.0, 0, 0], [0, 0, 1.0], [0, -1.0, 0]])   # disc normal along y
        for off in (cell_centers if cell_centers is not None else [(0.0, 0.0, 0.0)]):
            cells.append((shape @ rot.T + np.array([Lx / 2, 0.0, 0.0]) + np.asarray(off, float), f))
    wv = None
    if wall_vel is not None:
        n_layer = X.size
        wv = np.zeros((len(b2) * n_layer, 3), np.float32)
        wv[: wall_layers * n_layer] = wall_vel[0]
        wv[wall_layers * n_layer:] = wall_vel[1]
    b1a = np.concatenate(b1) if b1 else np.zeros((0, 3))
    return _assemble(name, bbox, 1 | 4, b1a, np.concatenate(b2), fluid, cells, phys, dx, wall_vel=wv)


def couette(nx=64, ny=32, nz=32, wall_layers=3, ncells=4, subdiv=3, cell_diameter=None, shear_rate=0.5,
            seed=12345, phys: Physics | None = None, name="couette") -> Config:
    """Couette flow for aggregation: the walls of `channel` move in -x and +x
    at -+U with U = shear_rate * Ly / 2 (prescribed through their VelHalf;
    the shear rate is in reduced units, 1/time), no body force, and `ncells`
    red cells stacked face to face across the channel (a rouleau: disc
    normals along y, centres 0.42 d apart), so that neighbouring membranes
    are within the Morse range.  The physics default turns aggregation on:
    De = 3e-3, beta = 1.5, r0 = 0.3, cut-off 2.5."""
    phys = phys or Physics(ext_force=0.0, sur_energy=3.0e-3, sca_fac=1.5, zero_len=0.3, max_cut=2.5)
    dx = 1.0 / 3.0
    Ly = ny * dx
    d = cell_diameter if cell_diameter is not None else min(8.0 / 1.5, 0.45 * ny * dx)
    u = shear_rate * Ly / 2.0
    pitch = 0.42 * d
    ys = (np.arange(ncells) - 0.5 * (ncells - 1)) * pitch
    centers = [(0.0, float(y), 0.0) for y in ys]
    if ncells and ((ncells - 1) * pitch + 0.35 * d > Ly - 2 * dx or d > min(nx, nz) * dx):
        raise ValueError("channel too small for the cells")
    return channel(nx=nx, ny=ny, nz=nz, wall_layers=wall_layers, b1_layers=0,
                   cell_subdiv=subdiv if ncells else -1, cell_diameter=d, seed=seed, phys=phys,
                   wall_vel=((-u, 0.0, 0.0), (u, 0.0, 0.0)), name=name,
                   cell_centers=centers if ncells else None)


def sheared_suspension(nx=136, ny=64, nz=136, wall_layers=3, ncells=64, subdiv=4, cell_diameter=None,
                       shear_rate=0.05, seed=12345, phys: Physics | None = None, max_tries=20000,
                       name="sheared_suspension") -> Config:
    """Red cells in Couette flow for rouleau tracking: the channel of `couette`
    (walls at y = -+Ly/2 moving at -+U, U = shear_rate * Ly / 2, no body
    force, Morse aggregation on) with `ncells` cells of 10*4^subdiv+2
    vertices at random positions and orientations, no two overlapping and
    each at least one lattice spacing from the walls; the fluid lattice
    sites nearest the membrane vertices are removed, one per vertex.  The
    default is 64 cells of 2562 vertices and 1,019,776 fluid particles
    (136 x 64 x 136 sites less 163,968).  The default diameter, 8, gives
    membrane edges of about 0.29 (0.87 dx); at the diameter of `channel`'s
    cell (5.33) a 2562-vertex membrane has edges of 0.19 and collapses
    within 500 steps at dt = 1e-3."""
    phys = phys or Physics(ext_force=0.0, sur_energy=3.0e-3, sca_fac=1.5, zero_len=0.3, max_cut=2.5)
    rng = np.random.default_rng(seed)
    dx = 1.0 / 3.0
    Lx, Ly, Lz = nx * dx, ny * dx, nz * dx
    d = cell_diameter if cell_diameter is not None else 8.0
    v_unit, faces = icosphere(subdiv)
    shape = biconcave(v_unit, d)
    body = rbc_body_points(d, dx * 0.9, 0.5 * dx)
    grid_n = np.array([int(Lx / dx), int(Ly / dx), int(Lz / dx)])
    occ = np.zeros(tuple(grid_n), bool)
    cells = []
    for _ in range(ncells):
        for _try in range(max_tries):
            R = random_rotation(rng)
            cen = rng.uniform(0, 1, 3) * np.array([Lx, Ly, Lz]) - np.array([0.0, Ly / 2, Lz / 2])
            verts = shape @ R.T + cen
            if np.abs(verts[:, 1]).max() > Ly / 2 - dx:
                continue
            pts = body @ R.T + cen
            idx = np.floor((pts + np.array([0.0, Ly / 2, Lz / 2])) / dx).astype(int)
            idx[:, 0] %= grid_n[0]
            idx[:, 2] %= grid_n[2]
            idx[:, 1] = np.clip(idx[:, 1], 0, grid_n[1] - 1)
            if occ[idx[:, 0], idx[:, 1], idx[:, 2]].any():
                continue
            occ[idx[:, 0], idx[:, 1], idx[:, 2]] = True
            cells.append((verts, faces))
            break
        else:
            raise RuntimeError(f"could not place cell {len(cells)} without overlap")
    base = couette(nx=nx, ny=ny, nz=nz, wall_layers=wall_layers, ncells=0, shear_rate=shear_rate, seed=seed,
                   phys=phys, name=name)
    fl0, fl1 = base.n_b1 + base.n_b2, base.n_b1 + base.n_b2 + base.n_fluid
    lattice = base.coor[fl0:fl1].astype(np.float64)
    ncp = sum(c[0].shape[0] for c in cells)
    if ncp:
        from scipy.spatial import cKDTree
        per = np.array([Lx, 2.0 * Ly + 1.0, Lz])   # x and z periodic; y far wider than the channel
        shift = np.array([0.0, Ly, Lz / 2])
        mv = np.mod(np.concatenate([c[0] for c in cells]) + shift, per)
        tree = cKDTree(mv, boxsize=per)
        dist, _ = tree.query(np.mod(lattice + shift, per), k=1, workers=-1)
        keep = np.argsort(dist, kind="stable")[ncp:]
        lattice = lattice[np.sort(keep)]
    b2 = base.coor[base.n_b1:fl0]
    cfg = _assemble(name, base.bbox, base.pmask, np.zeros((0, 3)), b2, lattice, cells, phys, dx,
                    wall_vel=base.velhalf[base.n_b1:fl0])
    cfg.meta = dict(ncells=ncells, diameter=d, shear_rate=shear_rate, wall_speed=shear_rate * Ly / 2.0, seed=seed)
    return cfg


def constriction(nx=96, ny=36, nz=24, wall_layers=3, b1_layers=1, ratio=2.0, ncells=2, subdiv=3,
                 cell_diameter=None, seed=12345, phys: Physics | None = None, name="constriction",
                 layout="line", max_tries=20000) -> Config:
    """Channel with a smooth 2:1 constriction of frozen wall particles: the
    walls y = +-h(x) follow the signed-distance profile
    h(x) = H - (H - H/ratio) (1 + cos(2 pi (x - Lx/2)/w))/2 for |x - Lx/2| < w/2
    (w = Lx/3) and H elsewhere, H = Ly/2.  Every lattice site of the box
    [0, Lx) x [-H - t, H + t) x [-Lz/2, Lz/2) (t = the wall thickness) with
    |y| < h(x) is fluid, h(x) <= |y| < h(x) + wall_layers dx is Bound2 and the
    next b1_layers dx is Bound1; the rest is empty.  Periodic in x and z;
    the body force drives the flow through the throat (the pressure drop of a
    driven inflow in a periodic channel).  layout "line": the cells sit in
    a row along z in the wide part, upstream of the throat, disc normals
    facing the flow; "random": at seeded random positions and orientations
    anywhere in the channel, no two overlapping and every vertex at least
    one lattice spacing inside the walls."""
    phys = phys or Physics()
    rng = np.random.default_rng(seed)
    dx = 1.0 / 3.0
    Lx, Ly, Lz = nx * dx, ny * dx, nz * dx
    H = Ly / 2
    t = (wall_layers + b1_layers) * dx
    w = Lx / 3.0

    def h(x):
        s = np.abs(x - Lx / 2)
        bump = 0.5 * (1 + np.cos(2 * np.pi * (x - Lx / 2) / w))
        return np.where(s < w / 2, H - (H - H / ratio) * bump, H)

    nyt = ny + 2 * (wall_layers + b1_layers)
    lat = _lattice(nx, nyt, nz, dx, (0.0, -H - t, -Lz / 2), rng)
    hx = h(lat[:, 0])
    ay = np.abs(lat[:, 1])
    fluid = lat[ay < hx]
    b2 = lat[(ay >= hx) & (ay < hx + wall_layers * dx)]
    b1 = lat[(ay >= hx + wall_layers * dx) & (ay < hx + t)]
    cells = []
    if ncells and layout == "random":
        d = cell_diameter if cell_diameter is not None else 8.0 / 1.5
        v, f = icosphere(subdiv)
        shape = biconcave(v, d)
        body = rbc_body_points(d, dx * 0.9, 0.5 * dx)
        grid_n = np.array([int(round(Lx / dx)), int(round(Ly / dx)), int(round(Lz / dx))])
        occ = np.zeros(tuple(grid_n), bool)
        off = np.array([0.0, H, Lz / 2])
        for _ in range(ncells):
            for _try in range(max_tries):
                R = random_rotation(rng)
                cen = rng.uniform(0, 1, 3) * np.array([Lx, Ly, Lz]) - np.array([0.0, H, Lz / 2])
                verts = shape @ R.T + cen
                if (np.abs(verts[:, 1]) > h(np.mod(verts[:, 0], Lx)) - dx).any():
                    continue
                idx = np.floor((body @ R.T + cen + off) / dx).astype(int)
                idx[:, 0] %= grid_n[0]
                idx[:, 2] %= grid_n[2]
                idx[:, 1] = np.clip(idx[:, 1], 0, grid_n[1] - 1)
                if occ[idx[:, 0], idx[:, 1], idx[:, 2]].any():
                    continue
                occ[idx[:, 0], idx[:, 1], idx[:, 2]] = True
                cells.append((verts, f))
                break
            else:
                raise RuntimeError(f"could not place cell {len(cells)} without overlap")
    elif ncells:
        d = cell_diameter if cell_diameter is not None else 0.5 * H
        v, f = icosphere(subdiv)
        shape = biconcave(v, d)
        rot = np.array([[0.0, 0, 1.0], [0, 1.0, 0], [-1.0, 0, 0]])   # disc normal along x (facing the flow)
        zs = (np.arange(ncells) - 0.5 * (ncells - 1)) * (1.1 * d)
        for z in zs:
            if abs(z) + 0.55 * d > Lz / 2:
                raise ValueError("box too thin for the cells")
            cells.append((shape @ rot.T + np.array([Lx / 6, 0.0, z]), f))
    if cells:
        from scipy.spatial import cKDTree
        per = np.array([Lx, 4.0 * (H + t) + 1.0, Lz])   # x and z periodic; y wider than the box
        shift = np.array([0.0, 2.0 * (H + t), Lz / 2])
        tree = cKDTree(np.mod(np.concatenate([c[0] for c in cells]) + shift, per), boxsize=per)
        dist, _ = tree.query(np.mod(fluid + shift, per), k=1, workers=-1)
        fluid = fluid[dist > 0.6 * dx]   # room for the membranes
    bbox = [0.0, Lx, -H - t, H + t, -Lz / 2, Lz / 2]
    return _assemble(name, bbox, 1 | 4, b1, b2, fluid, cells, phys, dx)


def rbc_body_points(diameter: float, spacing: float, margin: float) -> np.ndarray:
    """Grid points inside the biconcave shape dilated by `margin` (body frame)."""
    R = 0.5 * diameter + margin
    zmax = 0.2 * diameter + margin
    g = np.arange(-R, R + spacing, spacing)
    gz = np.arange(-zmax, zmax + spacing, spacing)
    X, Y, Z = np.meshgrid(g, g, gz, indexing="ij")
    rr = np.sqrt(X * X + Y * Y)
    s2 = np.clip((rr / (0.5 * diameter)) ** 2, 0.0, 1.0)
    half = diameter * np.sqrt(1.0 - s2) * (EF_A0 + EF_A1 * s2 / 4.0 + EF_A2 * s2 * s2 / 16.0)
    inside = (rr <= 0.5 * diameter + margin) & (np.abs(Z) <= half + margin)
    return np.stack([X[inside], Y[inside], Z[inside]], 1)


def unit_cell_volume(subdiv: int) -> float:
    """Volume of the biconcave cell of unit diameter (divergence theorem)."""
    v_unit, faces = icosphere(subdiv)
    shape = biconcave(v_unit, 1.0)
    a, b, c = (shape[faces[:, k]] for k in range(3))
    return float(np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6.0)


def suspension(nx=256, ny=128, nz=128, ncells=200, subdiv=4, hematocrit=0.20, seed=12345,
               phys: Physics | None = None, name="suspension", max_tries=20000, diameter=None) -> Config:
    """Periodic box of nx*ny*nz particles in total: `ncells` red cells of
    10*4^subdiv+2 vertices at random positions and orientations without
    overlap, the rest fluid on a jittered lattice with the lattice sites
    nearest the membranes removed.  The cell size follows from the
    hematocrit (cell volume fraction) unless `diameter` is given."""
    phys = phys or Physics(ext_force=0.0)
    rng = np.random.default_rng(seed)
    dx = 1.0 / 3.0
    L = np.array([nx, ny, nz], float) * dx
    v_unit, faces = icosphere(subdiv)
    unit_shape = biconcave(v_unit, 1.0)
    vol1 = unit_cell_volume(subdiv)
    box_vol = float(np.prod(L))
    if diameter is None:
        diameter = (hematocrit * box_vol / (ncells * vol1)) ** (1.0 / 3.0) if ncells else 0.0
    cells = []
    if ncells:
        shape = unit_shape * diameter
        h = dx
        grid_n = np.maximum((L / h).astype(int), 1)
        occ = np.zeros(tuple(grid_n), bool)
        body = rbc_body_points(diameter, h * 0.9, 0.5 * h)
        for _ in range(ncells):
            for _try in range(max_tries):
                R = random_rotation(rng)
                cen = rng.uniform(0, 1, 3) * L
                pts = body @ R.T + cen
                idx = np.floor(pts / h).astype(int) % grid_n
                if occ[idx[:, 0], idx[:, 1], idx[:, 2]].any():
                    continue
                occ[idx[:, 0], idx[:, 1], idx[:, 2]] = True
                cells.append((shape @ R.T + cen, faces))
                break
            else:
                raise RuntimeError(f"could not place cell {len(cells)} without overlap")
    lattice = _lattice(nx, ny, nz, dx, (0.0, 0.0, 0.0), rng)
    ncp = sum(c[0].shape[0] for c in cells)
    if ncp:
        from scipy.spatial import cKDTree
        mv = np.concatenate([c[0] for c in cells]) % L
        tree = cKDTree(mv, boxsize=L)
        dist, _ = tree.query(lattice % L, k=1, workers=-1)
        keep = np.argsort(dist, kind="stable")[ncp:]
        lattice = lattice[np.sort(keep)]
    return _assemble(name, [0.0, L[0], 0.0, L[1], 0.0, L[2]], 7, np.zeros((0, 3)), np.zeros((0, 3)), lattice,
                     cells, phys, dx)


def ensemble_suite(nsys=64, seed=2024, n_range=(8000, 200000), max_cells=16, subdiv=3, hct_max=0.30,
                   force_range=(2.0e-3, 5.0e-2), phys: Physics | None = None) -> list:
    """Independent periodic suspensions of uneven size for one ensemble: per
    system a particle count log-uniform in `n_range` (a 2:1:1 box of
    2 m^3 lattice sites), a hematocrit uniform in [0, hct_max] carried by 0
    to `max_cells` cells of 10*4^subdiv+2 vertices, a body force log-uniform
    in `force_range` and its own noise seed.  The cell diameter follows from
    the hematocrit and the cell count, at least 4.5 (so that the vertices
    of a 642-vertex membrane are about as far apart as the fluid particles,
    dx = 1/3) and at most 0.55 L_min (so that the cells fit the box); a box
    too small for such a cell gets none.  The hematocrit actually built is
    recorded in `cfg.meta` with the other draws.  Every system shares the
    remaining physical constants, as an ensemble requires."""
    base = phys or Physics()
    rng = np.random.default_rng(seed)
    dx = 1.0 / 3.0
    vol1 = unit_cell_volume(subdiv)
    out = []
    for s in range(nsys):
        n_target = float(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1]))))
        m = max(8, int(round((n_target / 2.0) ** (1.0 / 3.0))))
        hct = float(rng.uniform(0.0, hct_max))
        nc = int(rng.integers(0, max_cells + 1))
        g = float(np.exp(rng.uniform(np.log(force_range[0]), np.log(force_range[1]))))
        sub_seed = int(rng.integers(1, 2**31 - 1))
        ph = dataclasses.replace(base, ext_force=g, seed=sub_seed)
        box_vol = 2.0 * m ** 3 * dx ** 3
        lmin = m * dx
        d_min, d_max = 4.5, 0.55 * lmin
        if nc == 0 or hct < 0.01 or d_max < d_min:
            nc, d = 0, None
        else:
            d = (hct * box_vol / (nc * vol1)) ** (1.0 / 3.0)
            d = float(min(max(d, d_min), d_max))
        cfg = None
        while cfg is None:
            try:
                cfg = suspension(nx=2 * m, ny=m, nz=m, ncells=nc, subdiv=subdiv, seed=sub_seed, phys=ph,
                                 name=f"ensemble{s}", diameter=d, max_tries=4000)
            except RuntimeError:   # no room left for a cell: make the cells smaller, then fewer
                if d > d_min:
                    d = max(d_min, 0.9 * d)
                else:
                    nc -= 1
        built = nc * vol1 * d ** 3 / box_vol if nc else 0.0
        cfg.meta = dict(system=s, lattice=(2 * m, m, m), ncells=nc, diameter=d or 0.0, hematocrit=built,
                        hematocrit_drawn=hct, ext_force=g, seed=sub_seed)
        out.append(cfg)
    return out


def small_channel(seed=7, with_cell=True, b1_layers=1, nx=24, ny=12, nz=12, subdiv=2, diameter=3.0,
                  phys: Physics | None = None) -> Config:
    """A few-thousand-particle channel for parity tests (all particle types)."""
    return channel(nx=nx, ny=ny, nz=nz, wall_layers=3, b1_layers=b1_layers, cell_subdiv=subdiv if with_cell else -1,
                   cell_diameter=diameter, seed=seed, phys=phys, name="small_channel")


# ---------------------------------------------------------------------------
# GPUCell's four input files (src/Particle.cu:45-427): 20-character columns
# ---------------------------------------------------------------------------

def _row(vals) -> str:
    return "".join(f"{v:<20}" if isinstance(v, (int, np.integer)) else f"{float(v):<20.9g}" for v in vals) + "\n"


def write_reference_inputs(cfg: Config, directory: str) -> None:
    """Writes SDPDParCoor.txt, SDPDPhyPara.txt, CELLParStruct.txt and
    CELLPhyPara.txt as GPUCell's loaders read them."""
    os.makedirs(directory, exist_ok=True)
    p = cfg.phys
    with open(os.path.join(directory, "SDPDParCoor.txt"), "w") as f:
        f.write("nBound1 nBound2 nFluid\n")
        f.write(_row([cfg.n_b1, cfg.n_b2, cfg.n_fluid]))
        off = 0
        for label, cnt in (("Bound1", cfg.n_b1), ("Bound2", cfg.n_b2), ("Fluid", cfg.n_fluid)):
            f.write(f"{label} x y z\n")
            for x in cfg.coor[off:off + cnt]:
                f.write(_row(x))
            off += cnt
    with open(os.path.join(directory, "SDPDPhyPara.txt"), "w") as f:
        f.write("SoundSpeed1 / SoundSpeed2\n")
        f.write(_row([p.sound1]))
        f.write(_row([p.sound2]))
        f.write("ShearVis\n" + _row([p.shear_vis]))
        f.write("BulkVis\n" + _row([p.bulk_vis]))
        f.write("DenInit\n" + _row([cfg.den_init]))
        f.write("ConstExtForce (per unit mass)\n" + _row([p.ext_force]))
    with open(os.path.join(directory, "CELLParStruct.txt"), "w") as f:
        f.write("nCell\n" + _row([cfg.ncell]))
        ncs = cfg.n_cell_start
        voff = toff = eoff = 0
        for c in range(cfg.ncell):
            nv, nt = int(cfg.npar[c]), int(cfg.ntri_cell[c])
            ne = nt * 3 // 2
            f.write("Type nPar nTri nEdgeInfo\n" + _row([int(cfg.cell_type[c]), nv, nt, 6]))
            f.write("x y z\n")
            for x in cfg.coor[ncs + voff: ncs + voff + nv]:
                f.write(_row(x))
            f.write("v1 v2 v3\n")
            for t in cfg.tri[toff:toff + nt]:
                f.write(_row([int(t[0]) - voff, int(t[1]) - voff, int(t[2]) - voff]))
            f.write("p1 p2 p3 p4 t1 t2\n")
            for e in cfg.edge[eoff:eoff + ne]:
                f.write(_row([int(e[0]) - voff, int(e[1]) - voff, int(e[2]) - voff, int(e[3]) - voff,
                              int(e[4]) - toff, int(e[5]) - toff]))
            voff += nv
            toff += nt
            eoff += ne
    with open(os.path.join(directory, "CELLPhyPara.txt"), "w") as f:
        f.write("nType\n" + _row([1]))
        f.write("ShearMod\n" + _row([p.shear_mod]))
        f.write("BendingMod\n" + _row([p.bending_mod]))
        f.write("HGarea\n" + _row([p.hgarea]))
        f.write("HLarea\n" + _row([p.hlarea]))
        f.write("HVol\n" + _row([p.hvol]))
        f.write("MaxCut\n" + _row([p.max_cut]))
        f.write("zeroLen\n" + _row([p.zero_len]))
        f.write("scaFac\n" + _row([p.sca_fac]))
        f.write("surEnergy\n" + _row([p.sur_energy]))


def _col(line: str, k: int) -> str:
    return line[20 * k: 20 * k + 20]


def read_reference_inputs(directory: str) -> dict:
    """Parses the four files with the reference's rules (fixed 20-character
    columns, atoi/atof semantics, per-cell offsets added to the topology)."""
    def lines(name):
        with open(os.path.join(directory, name)) as f:
            return f.read().split("\n")

    out = {}
    L = lines("SDPDParCoor.txt")
    nb1, nb2, nfl = (int(float(_col(L[1], k))) for k in range(3))
    pos, r = [], 2
    for cnt in (nb1, nb2, nfl):
        r += 1
        for _ in range(cnt):
            pos.append([float(_col(L[r], k)) for k in range(3)])
            r += 1
    out.update(n_b1=nb1, n_b2=nb2, n_fluid=nfl, sdpd_coor=np.asarray(pos, np.float32).reshape(-1, 3))
    L = lines("SDPDPhyPara.txt")
    out.update(sound1=float(_col(L[1], 0)), sound2=float(_col(L[2], 0)), shear_vis=float(_col(L[4], 0)),
               bulk_vis=float(_col(L[6], 0)), den_init=float(_col(L[8], 0)), ext_force=float(_col(L[10], 0)))
    L = lines("CELLParStruct.txt")
    ncell = int(float(_col(L[1], 0)))
    r = 2
    coor, tri, edge, betri, celltab = [], [], [], [], []
    a = b = m = 0
    for c in range(ncell):
        r += 1
        npar, ntri = int(float(_col(L[r], 1))), int(float(_col(L[r], 2)))
        r += 2
        for _ in range(npar):
            coor.append([float(_col(L[r], k)) for k in range(3)])
            celltab.append(c)
            r += 1
        r += 1
        betri.append([m, m + ntri - 1])
        for _ in range(ntri):
            tri.append([int(float(_col(L[r], k))) + b for k in range(3)])
            r += 1
            m += 1
        r += 1
        for _ in range(ntri * 3 // 2):
            e = [int(float(_col(L[r], k))) for k in range(6)]
            edge.append([e[0] + b, e[1] + b, e[2] + b, e[3] + b, e[4] + a, e[5] + a])
            r += 1
        a += ntri
        b += npar
    out.update(ncell=ncell, cell_coor=np.asarray(coor, np.float32).reshape(-1, 3),
               tri=np.asarray(tri, np.int32).reshape(-1, 3), edge=np.asarray(edge, np.int32).reshape(-1, 6),
               betri=np.asarray(betri, np.int32).reshape(-1, 2), celltab=np.asarray(celltab, np.int32))
    return out
