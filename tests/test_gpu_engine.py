"""GPUCell's own call sequence with the fused engine behind it.

`ParticleSystem` calls the 20 boundary entry points exactly as
Particle::UpdatePar does; with gc_set_engine(1) every step after the first
runs fused inside SetFluidExtForce and writes back what the host reads.
Compared with the entry-point kernels on the same sequence (noise on, so the
same Philox pair noise): positions within 1e-5, velocities and forces within
1e-4 of their largest magnitude, densities within 1e-5 relative (the fused
step's double-float positions differ from the entry points' FP32 positions
by up to an FP32 ulp per step, 1.3e-6 relative in density after 4 steps),
membrane outputs within 1e-5 relative.
"""
import numpy as np
import pytest

from gpucell_gb300 import generator as gen

pytestmark = pytest.mark.gpu


@pytest.fixture
def engine_mode():
    from gpucell_gb300 import _lib
    yield lambda m: _lib.call("gc_set_engine", m)
    _lib.call("gc_set_engine", 0)


def _close_rel(got, want, tol):
    scale = max(np.abs(want).max(), 1e-30)
    assert np.abs(got - want).max() <= tol * scale


def _run(cfg, mode, engine_mode, steps, noise=True):
    from gpucell_gb300.host import ParticleSystem
    engine_mode(mode)
    ps = ParticleSystem(cfg, noise=noise)
    for _ in range(steps):
        ps.update()
    out = ps.fetch()
    del ps
    return out


@pytest.mark.parametrize("name", ["channel", "suspension", "two_cells"])
def test_engine_follows_entry_point_kernels(cuda_device, engine_mode, name):
    if name == "channel":
        cfg = gen.small_channel()
    elif name == "suspension":
        cfg = gen.suspension(nx=36, ny=24, nz=24, ncells=3, subdiv=2, hematocrit=0.15, seed=3)
    else:
        phys = gen.Physics(sur_energy=5.0, max_cut=1.2, zero_len=0.3, sca_fac=4.0)
        cfg = gen.channel(nx=24, ny=12, nz=18, wall_layers=3, b1_layers=1, cell_subdiv=2, cell_diameter=3.0,
                          phys=phys, cell_centers=[(0.0, -0.55, 0.0), (0.0, 0.55, 0.0)], seed=11)
    a = _run(cfg, 0, engine_mode, 4)
    b = _run(cfg, 1, engine_mode, 4)
    np.testing.assert_allclose(b["pos"], a["pos"], atol=1e-5)
    _close_rel(b["vel"], a["vel"], 1e-4)
    _close_rel(b["force"], a["force"], 1e-4)
    _close_rel(b["rho"], a["rho"], 1e-5)
    assert np.array_equal(b["nthro"], a["nthro"])
    # the host's view: SortPart is a permutation and CurPos its inverse
    assert np.array_equal(np.sort(b["sortpart"]), np.arange(cfg.n))
    np.testing.assert_allclose(b["Area"], a["Area"], rtol=1e-5)
    np.testing.assert_allclose(b["Vol"], a["Vol"], rtol=1e-5)
    np.testing.assert_allclose(b["TriNorDir"], a["TriNorDir"], atol=1e-4)
    np.testing.assert_allclose(b["TriCenter"], a["TriCenter"], atol=1e-4)
    edge = float(np.mean(a["RefEdgeLen"]))
    np.testing.assert_allclose(b["DefForce"], a["DefForce"], atol=1e-5 * cfg.phys.hgarea * edge)
    _close_rel(b["AggForce"], a["AggForce"], 1e-4) if np.abs(a["AggForce"]).max() > 0 else None
