"""The pair tiles of the fused step (GcFusedOptions.tiles: half-stencil
passes, every pair once, each side its share, sums in a fixed order) against
the per-particle list passes and the FP64 oracle.

Tolerances, stated per test:
  * a few steps from the same state, noise off: positions within 1e-5 of
    the oracle, forces per particle within 1e-5 |F_i| + 16 u S_i (u FP32's
    unit roundoff, S_i the sum of the magnitudes of the terms F_i adds up,
    the pressure counted at c^2 rho since it amplifies the density's
    rounding); tiles and lists within the same bounds of each other;
  * two runs of the same input, noise on, across list rebuilds:
    bit-identical (the lanes that add to one particle in the same iteration
    take turns in an order fixed when the lists are built);
  * a cube holding more particles than the tiles take: the handle turns to
    per-particle lists by itself and steps as a handle created with them
    (bit-identical), host-driven and in captured steps.
"""
import numpy as np
import pytest

from gpucell_gb300 import generator as gen

pytestmark = pytest.mark.gpu


def _oracle(cfg, noise):
    from oracle.binding import Oracle
    o = Oracle(cfg, noise=noise)
    o.setup()
    return o


def _configs():
    phys = gen.Physics(sur_energy=5.0, max_cut=1.2, zero_len=0.3, sca_fac=4.0)
    return {
        # periodic on all axes, cells across the faces
        "suspension": gen.suspension(nx=36, ny=24, nz=24, ncells=3, subdiv=2, hematocrit=0.15, seed=3),
        # Bound1 and Bound2 walls in y, a cell
        "channel": gen.small_channel(),
        # moving Bound2 walls, two cells with Morse aggregation
        "couette": gen.couette(nx=36, ny=18, nz=24, ncells=2, subdiv=2, cell_diameter=3.0, shear_rate=0.5, seed=31,
                               phys=phys),
    }


@pytest.mark.parametrize("name", ["suspension", "channel", "couette"])
def test_tiles_match_lists_and_the_oracle(cuda_device, name):
    from gpucell_gb300.fused import FusedSystem
    from oracle.binding import force_error_stats
    cfg = _configs()[name]
    tiles = FusedSystem(cfg, noise=False, tiles=True)
    lists = FusedSystem(cfg, noise=False)
    assert tiles.options()["tiles"] is True and lists.options()["tiles"] is False
    o = _oracle(cfg, False)
    for _ in range(3):
        o.step()
    tiles.step(3, 1)
    lists.step(3, 1)
    t, li = tiles.fetch(), lists.fetch()
    assert tiles.flags() == 0 and lists.flags() == 0
    np.testing.assert_allclose(t["pos"], o.pos, atol=1e-5)
    np.testing.assert_allclose(t["pos"], li["pos"], atol=1e-5)
    mov = slice(cfg.n_b1 + cfg.n_b2, cfg.n)
    scale = o.force_scale()[mov]
    st = force_error_stats(t["force"][mov], o.force[mov], scale)
    sl = force_error_stats(li["force"][mov], o.force[mov], scale)
    print(f"\n{name}: tiles median rel {st['median_rel']:.2e} p99 {st['p99_rel']:.2e} worst/bound "
          f"{st['worst_ratio']:.3f}; lists median rel {sl['median_rel']:.2e} p99 {sl['p99_rel']:.2e} worst/bound "
          f"{sl['worst_ratio']:.3f}; mean neighbours {tiles.stats()['mean_neighbors']:.1f}")
    assert st["worst_ratio"] <= 1.0 and sl["worst_ratio"] <= 1.0
    np.testing.assert_allclose(t["rho"][mov], o.rho[mov], rtol=1e-5)
    if cfg.ncell:
        np.testing.assert_allclose(t["Area64"], o.area, rtol=1e-5)
        np.testing.assert_allclose(t["Vol64"], o.vol, rtol=1e-5)
    if cfg.phys.sur_energy:
        assert np.abs(o.aggforce).max() > 0
    tiles.close()
    lists.close()


@pytest.mark.parametrize("graph", [False, True])
def test_tiles_are_bit_reproducible(cuda_device, graph):
    """Every shared-memory sum is added in an order fixed by the lists, so
    the run is the same every time."""
    from gpucell_gb300.fused import FusedSystem
    cfg = gen.suspension(nx=32, ny=24, nz=24, ncells=2, subdiv=2, hematocrit=0.1, seed=9)
    runs = []
    for _ in range(2):
        fs = FusedSystem(cfg, noise=True, skin=0.02, graph=graph, tiles=True)
        fs.step(25, 1)
        runs.append(fs.fetch())
        assert fs.stats()["rebuilds"] >= 3 and fs.flags() == 0
        fs.close()
    for k in ("pos", "vel", "force", "rho", "Area64", "Vol64"):
        assert np.array_equal(runs[0][k], runs[1][k]), k


def _crowded(seed=4, skin=0.1):
    """A periodic fluid box (8 rc wide, 7 cubes of rc + skin per axis) with
    130 fluid particles gathered 0.16 rc apart inside the middle of one cube:
    with the ~33 already there, more than the 96 the pair tiles take."""
    import dataclasses
    cfg = gen.suspension(nx=24, ny=24, nz=24, ncells=0, seed=seed)
    coor = cfg.coor.copy()
    rng = np.random.default_rng(seed)
    lo = cfg.bbox[0::2].astype(np.float64)
    L = cfg.bbox[1::2].astype(np.float64) - lo
    ncube = np.floor(L / ((1.0 + skin) * (1.0 + 1e-4)))
    centre = lo + 3.5 * L / ncube
    pick = rng.choice(np.arange(cfg.n_b1 + cfg.n_b2, cfg.n_cell_start), 130, replace=False)
    g = np.stack(np.meshgrid(*[np.arange(6)] * 3, indexing="ij"), -1).reshape(-1, 3)[:130]
    coor[pick] = (centre - 0.4 + 0.16 * g + rng.uniform(-0.005, 0.005, size=(130, 3))).astype(np.float32)
    return dataclasses.replace(cfg, coor=coor)


@pytest.mark.parametrize("graph", [False, True])
def test_tiles_fall_back_to_lists_for_a_crowded_cube(cuda_device, graph):
    from gpucell_gb300.fused import FusedSystem
    cfg = _crowded()
    fs = FusedSystem(cfg, noise=False, graph=graph, tiles=True)
    ref = FusedSystem(cfg, noise=False, graph=graph)
    fs.step(3, 1)
    ref.step(3, 1)
    assert fs.options()["tiles"] is False      # turned to lists by itself
    a, b = fs.fetch(), ref.fetch()
    for k in ("pos", "vel", "force", "rho"):
        assert np.array_equal(a[k], b[k]), k
    assert np.isfinite(a["force"]).all()
    fs.close()
    ref.close()
