"""Synthetic inputs: mesh topology and GPUCell's input-file format (no GPU)."""
import numpy as np

from gpucell_gb300 import generator as gen


def test_icosphere_counts_and_edges():
    for s, nv in ((2, 162), (3, 642), (4, 2562)):
        v, f = gen.icosphere(s)
        assert v.shape == (nv, 3) and f.shape == (2 * nv - 4, 3)
        e = gen.edge_records(f)
        assert e.shape[0] == f.shape[0] * 3 // 2          # src/Particle.cu:217
        # p1 -> p2 runs forward in t1 and backward in t2; p3/p4 are the third vertices
        for p1, p2, p3, p4, t1, t2 in e[:200]:
            a, b = list(f[t1]), list(f[t2])
            assert set(a) == {p1, p2, p3} and set(b) == {p1, p2, p4}
            i = a.index(p1)
            assert a[(i + 1) % 3] == p2
            j = b.index(p2)
            assert b[(j + 1) % 3] == p1


def test_channel_counts_match_configuration():
    cfg = gen.channel()
    assert (cfg.n_fluid, cfg.n_b2, cfg.ncp, cfg.ntri, cfg.nedge) == (65536, 12288, 642, 1280, 1920)
    c = cfg.consts()
    assert c["nCellStart"] + c["nCellPar"] == c["nTotalPar"] == cfg.n


def test_reference_file_round_trip(tmp_path):
    cfg = gen.small_channel()
    gen.write_reference_inputs(cfg, str(tmp_path))
    got = gen.read_reference_inputs(str(tmp_path))
    assert (got["n_b1"], got["n_b2"], got["n_fluid"]) == (cfg.n_b1, cfg.n_b2, cfg.n_fluid)
    np.testing.assert_allclose(got["sdpd_coor"], cfg.coor[:cfg.n_cell_start], rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(got["cell_coor"], cfg.coor[cfg.n_cell_start:], rtol=1e-6, atol=1e-6)
    np.testing.assert_array_equal(got["tri"], cfg.tri)
    np.testing.assert_array_equal(got["edge"], cfg.edge)
    np.testing.assert_array_equal(got["betri"], cfg.betri)
    np.testing.assert_array_equal(got["celltab"], cfg.celltab)
    assert abs(got["den_init"] - cfg.den_init) < 1e-6 * cfg.den_init
    # every line fits the reference's 200-character line buffer (src/Particle.cu:50)
    for name in ("SDPDParCoor.txt", "SDPDPhyPara.txt", "CELLParStruct.txt", "CELLPhyPara.txt"):
        assert max(len(ln) for ln in open(tmp_path / name)) < 200


def test_suspension_small_has_no_overlap_and_exact_count():
    cfg = gen.suspension(nx=48, ny=32, nz=32, ncells=3, subdiv=2, hematocrit=0.1)
    assert cfg.n == 48 * 32 * 32
    assert cfg.ncp == 3 * 162 and cfg.pmask == 7


def test_reference_grid_formula():
    from gpucell_gb300.host import reference_grid
    ncube, outer, invwid, size = reference_grid([0, 20, -10, 10, -10, 10])   # src/main.cuh:12
    assert ncube == [20, 22, 22] and outer == [20.0, 22.0, 22.0] and size == 9680


def test_ensemble_suite_draws_within_the_stated_ranges():
    cfgs = gen.ensemble_suite(nsys=8, seed=3, n_range=(8000, 60000), max_cells=4, subdiv=1)
    assert len(cfgs) == 8
    ref = cfgs[0].consts()
    fixed = [k for k in ref if k not in ("nBound2Start", "nFluidStart", "nCellStart", "nTotalPar", "nCellPar",
                                         "iSeed", "ConstExtForce")]
    seeds = set()
    for c in cfgs:
        m = c.meta
        assert 8000 * 0.8 <= c.n <= 60000 * 1.2 and c.pmask == 7
        assert 0 <= m["ncells"] <= 4 and c.ncell == m["ncells"] and c.ncp == 42 * m["ncells"]
        assert 0.0 <= m["hematocrit"] <= 0.30 + 1e-9
        assert 2.0e-3 <= m["ext_force"] <= 5.0e-2
        k = c.consts()
        assert all(k[f] == ref[f] for f in fixed)   # one ensemble: same physics
        seeds.add(k["iSeed"])
    assert len(seeds) == 8
    again = gen.ensemble_suite(nsys=8, seed=3, n_range=(8000, 60000), max_cells=4, subdiv=1)
    assert all(np.array_equal(a.coor, b.coor) for a, b in zip(cfgs, again))


def test_couette_walls_move_and_cells_touch():
    cfg = gen.couette(nx=36, ny=18, nz=18, ncells=2, subdiv=2, cell_diameter=3.0, shear_rate=0.5)
    u = 0.5 * (18 / 3.0) / 2
    b2 = cfg.velhalf[cfg.n_b1:cfg.n_b1 + cfg.n_b2]
    y = cfg.coor[cfg.n_b1:cfg.n_b1 + cfg.n_b2, 1]
    assert np.allclose(b2[y < 0, 0], -u) and np.allclose(b2[y > 0, 0], u)
    assert np.all(cfg.velhalf[cfg.n_b1 + cfg.n_b2:] == 0)
    c = cfg.consts()
    assert c["ConstExtForce"] == 0 and c["surEnergy"] > 0 and c["MaxCut"] == 2.5
    m = cfg.coor[cfg.n_cell_start:].astype(np.float64)
    a, b = m[:162], m[162:]
    gap = np.sqrt(((a[:, None, :] - b[None, :, :]) ** 2).sum(-1)).min()
    assert 0.0 < gap < c["MaxCut"]


def test_constriction_walls_follow_the_profile():
    cfg = gen.constriction(nx=48, ny=24, nz=18, ncells=2, subdiv=2, cell_diameter=2.4)
    H = 24 / 3.0 / 2
    fl = cfg.coor[cfg.n_b1 + cfg.n_b2:cfg.n_cell_start]
    x, y = fl[:, 0], np.abs(fl[:, 1])
    Lx = 48 / 3.0
    throat = np.abs(x - Lx / 2) < 0.2
    wide = x < Lx / 6 - 1.5
    assert y[throat].max() < 0.52 * H and y[wide].max() > 0.9 * H   # 2:1
    b2 = cfg.coor[cfg.n_b1:cfg.n_b1 + cfg.n_b2]
    assert np.abs(b2[np.abs(b2[:, 0] - Lx / 2) < 0.2, 1]).min() >= 0.49 * H
    assert cfg.n_b1 > 0 and cfg.ncell == 2 and cfg.pmask == 5


def test_sheared_suspension_places_cells_inside_the_channel():
    cfg = gen.sheared_suspension(nx=36, ny=24, nz=36, ncells=6, subdiv=2, cell_diameter=3.0, shear_rate=0.5, seed=3)
    Ly = 24 / 3.0
    assert cfg.ncell == 6 and cfg.ncp == 6 * 162
    assert cfg.n_fluid == 36 * 24 * 36 - cfg.ncp          # one lattice site removed per vertex
    m = cfg.coor[cfg.n_cell_start:].astype(np.float64)
    assert np.abs(m[:, 1]).max() <= Ly / 2 - 1.0 / 3.0   # clear of the walls
    u = 0.5 * Ly / 2
    b2 = cfg.velhalf[cfg.n_b1:cfg.n_b1 + cfg.n_b2]
    y = cfg.coor[cfg.n_b1:cfg.n_b1 + cfg.n_b2, 1]
    assert np.allclose(b2[y < 0, 0], -u) and np.allclose(b2[y > 0, 0], u)
    # no two cells overlap: their vertices stay apart (periodic in x and z)
    L = np.array([36 / 3.0, np.inf, 36 / 3.0])
    for a in range(6):
        for b in range(a + 1, 6):
            d = m[162 * a:162 * (a + 1), None, :] - m[None, 162 * b:162 * (b + 1), :]
            d[..., [0, 2]] -= L[[0, 2]] * np.rint(d[..., [0, 2]] / L[[0, 2]])
            assert np.sqrt((d ** 2).sum(-1)).min() > 0.2
