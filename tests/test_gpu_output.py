"""Output files written from the fused step (gc_ensemble_write_output).

* The per-cell statistics reduced on the GPU in FP64 equal the means of the
  stored per-vertex arrays (relative 1e-6): mean DefForce and AggForce,
  mean velocity and its magnitude, area and volume.
* The written files read back to the stored state within the 6 significant
  digits of the format (relative 1e-5), per type zone, and the cell zones
  reproduce the membrane topology.
* One system of an ensemble writes the same files as the system run alone
  would, up to the summation order of the other systems' rebuilds.
"""
import os

import numpy as np
import pytest

from gpucell_gb300 import generator as gen
from gpucell_gb300.output import read_plt

pytestmark = pytest.mark.gpu


PHYS = gen.Physics(sur_energy=5.0, max_cut=1.2, zero_len=0.3, sca_fac=4.0)


def _cfg():
    phys = PHYS
    return gen.channel(nx=24, ny=12, nz=18, wall_layers=3, b1_layers=1, cell_subdiv=2, cell_diameter=3.0,
                       phys=phys, cell_centers=[(0.0, -0.55, 0.0), (0.0, 0.55, 0.0)], seed=11)


def _means(cfg, got):
    out = np.zeros((cfg.ncell, 12))
    v0 = 0
    for c in range(cfg.ncell):
        nv = int(cfg.npar[c])
        sl = slice(v0, v0 + nv)
        out[c, 0:3] = got["DefForce"][sl].astype(np.float64).mean(0)
        out[c, 3:6] = got["AggForce"][sl].astype(np.float64).mean(0)
        out[c, 6:9] = got["vel"][cfg.n_cell_start + v0:cfg.n_cell_start + v0 + nv].astype(np.float64).mean(0)
        out[c, 9] = np.linalg.norm(out[c, 6:9])
        out[c, 10], out[c, 11] = got["Area64"][c], got["Vol64"][c]
        v0 += nv
    return out


def test_cell_stats_and_files(cuda_device, tmp_path):
    from gpucell_gb300.fused import FusedSystem
    cfg = _cfg()
    fs = FusedSystem(cfg, noise=True)
    fs.step(6, 1)
    got = fs.fetch()
    st = fs.cell_stats()
    want = _means(cfg, got)
    assert np.abs(want[:, 3:6]).max() > 0       # the aggregation force acts
    np.testing.assert_allclose(st, want, rtol=1e-6, atol=1e-12 * np.abs(want).max())
    d = str(tmp_path / "Result")
    fs.write_output(d, 6, 0.006, first=True)
    coor = read_plt(os.path.join(d, "FluidCoor", "6.plt"))
    bounds = [0, cfg.n_b1, cfg.n_b1 + cfg.n_b2, cfg.n_cell_start, cfg.n]
    assert len(coor) == 4
    for z, (lo, hi) in zip(coor, zip(bounds[:-1], bounds[1:])):
        np.testing.assert_allclose(z["rows"][:, :3], got["pos"][lo:hi], rtol=1e-5, atol=1e-6)
        np.testing.assert_array_equal(z["rows"][:, 3], np.arange(lo, hi))
    field = read_plt(os.path.join(d, "FluidField", "6.plt"))[0]["rows"]
    cs = cfg.n_cell_start
    np.testing.assert_allclose(field[:, 3], got["rho"][:cs], rtol=1e-5)
    np.testing.assert_allclose(field[:, 5:8], got["vel"][:cs], rtol=1e-5, atol=1e-6 * np.abs(got["vel"]).max())
    cells = read_plt(os.path.join(d, "CellForce", "6.plt"))
    assert len(cells) == cfg.ncell
    v0 = 0
    for c, z in enumerate(cells):
        nv = int(cfg.npar[c])
        assert z["header"] == f"Zone N={nv}, E={int(cfg.ntri_cell[c])}, F=FEPOINT, ET=TRIANGLE"
        np.testing.assert_allclose(z["rows"][:, 3:6], got["DefForce"][v0:v0 + nv], rtol=1e-5,
                                   atol=1e-6 * np.abs(got["DefForce"]).max())
        t0, t1 = cfg.betri[c]
        np.testing.assert_array_equal(z["conn"], cfg.tri[t0:t1 + 1] - v0)
        v0 += nv
    tf = np.loadtxt(os.path.join(d, "CellForce", "TF_Cell1.plt"), ndmin=2)
    np.testing.assert_allclose(tf[0, 1:7], st[1, :6], rtol=1e-5)
    geo = np.loadtxt(os.path.join(d, "CellGeo", "Geo_Cell0.plt"), ndmin=2)
    np.testing.assert_allclose(geo[0], [0.006, st[0, 9], st[0, 10], st[0, 11]], rtol=1e-5)
    nd = read_plt(os.path.join(d, "CellNorDir", "6.plt"))
    np.testing.assert_allclose(np.concatenate([z["rows"][:, 3:6] for z in nd]), got["TriNorDir"], rtol=1e-5,
                               atol=1e-6)


def test_ensemble_system_writes_its_own_files(cuda_device, tmp_path):
    from gpucell_gb300.fused import Ensemble
    a = gen.suspension(nx=16, ny=16, nz=16, ncells=0, seed=5, phys=PHYS)
    b = _cfg()
    ens = Ensemble([a, b], noise=False)
    ens.step(3, 1)
    d = str(tmp_path / "Result")
    ens.write_output(d, 3, 0.003, first=True, sys=1)
    got = ens.fetch(1)
    field = read_plt(os.path.join(d, "FluidField", "3.plt"))[0]["rows"]
    assert field.shape[0] == b.n_cell_start
    np.testing.assert_allclose(field[:, :3], got["pos"][:b.n_cell_start], rtol=1e-5, atol=1e-6)
    assert len(read_plt(os.path.join(d, "CellCoor", "3.plt"))) == b.ncell


def test_system_without_cells_writes_its_files(cuda_device, tmp_path):
    """A system without membranes writes the particle files (and no cell
    files or series) without error."""
    from gpucell_gb300.fused import FusedSystem
    from gpucell_gb300.output import read_plt
    cfg = gen.suspension(nx=16, ny=16, nz=16, ncells=0, seed=5)
    fs = FusedSystem(cfg, noise=True)
    fs.step(3, 1)
    d = str(tmp_path / "Result")
    fs.write_output(d, 3, 0.003, first=True)
    zones = read_plt(os.path.join(d, "FluidCoor", "3.plt"))
    assert sum(z["rows"].shape[0] for z in zones) == cfg.n
    assert not os.path.exists(os.path.join(d, "CellCoor", "3.plt"))
    fs.close()
