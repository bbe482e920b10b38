"""The fused timestep (gc_fused_*) against the FP64 oracle and against the
boundary entry points.

Tolerances, stated per test:
  * a few steps from rest, noise off: positions within 1e-5, velocities
    within 1e-4 of their largest magnitude, cell area and volume (FP64 sums)
    within 1e-5 relative of the oracle;
  * noise on, against the boundary entry points (same Philox pair noise):
    positions within 1e-5, forces within 1e-4 of their largest magnitude.
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


def _close_rel(got, want, tol):
    scale = max(np.abs(want).max(), 1e-30)
    err = np.abs(got - want).max()
    assert err <= tol * scale, f"max err {err:g} vs scale {scale:g}"


# the per-particle lists (default) with and without the per-step compaction
# of the acting entries, and the pair tiles
MODES = {"lists_compact": dict(compact=True), "lists": dict(compact=False), "tiles": dict(tiles=True)}


@pytest.mark.parametrize("mode", list(MODES))
def test_fused_tracks_oracle_noise_off(cuda_device, mode):
    from gpucell_gb300.fused import FusedSystem
    cfg = gen.small_channel()
    fs = FusedSystem(cfg, noise=False, **MODES[mode])
    o = _oracle(cfg, False)
    for _ in range(3):
        fs.step(1, 1)
        o.step()
    g = fs.fetch()
    np.testing.assert_allclose(g["pos"], o.pos, atol=1e-5)
    _close_rel(g["vel"], o.vel, 1e-4)
    np.testing.assert_allclose(g["Area64"], o.area, rtol=1e-5)
    np.testing.assert_allclose(g["Vol64"], o.vol, rtol=1e-5)
    np.testing.assert_allclose(g["rho"][cfg.n_b1 + cfg.n_b2:], o.rho[cfg.n_b1 + cfg.n_b2:], rtol=1e-5)
    assert fs.flags() == 0


@pytest.mark.parametrize("mode", list(MODES))
def test_fused_matches_boundary_path_with_noise(cuda_device, mode):
    from gpucell_gb300.fused import FusedSystem
    from gpucell_gb300.host import ParticleSystem
    cfg = gen.small_channel()
    ps = ParticleSystem(cfg, noise=True)
    fs = FusedSystem(cfg, noise=True, **MODES[mode])
    for _ in range(2):
        ps.update()
        fs.step(1, 1)
    a, b = ps.fetch(), fs.fetch()
    np.testing.assert_allclose(b["pos"], a["pos"], atol=1e-5)
    _close_rel(b["force"], a["force"], 1e-4)
    _close_rel(b["vel"], a["vel"], 1e-4)


def test_fused_rebuilds_keep_parity(cuda_device):
    """A tiny skin forces frequent list rebuilds; the trajectory still
    follows the oracle (noise off)."""
    from gpucell_gb300.fused import FusedSystem
    cfg = gen.small_channel()
    fs = FusedSystem(cfg, noise=False, skin=0.002)
    o = _oracle(cfg, False)
    for _ in range(8):
        fs.step(1, 1)
        o.step()
    st = fs.stats()
    assert st["rebuilds"] >= 3, st
    g = fs.fetch()
    np.testing.assert_allclose(g["pos"], o.pos, atol=5e-5)
    _close_rel(g["vel"], o.vel, 1e-3)


def test_fused_periodic_suspension(cuda_device):
    """Fully periodic box with cells that cross the faces."""
    from gpucell_gb300.fused import FusedSystem
    cfg = gen.suspension(nx=36, ny=24, nz=24, ncells=3, subdiv=2, hematocrit=0.15, seed=3)
    fs = FusedSystem(cfg, noise=False)
    o = _oracle(cfg, False)
    for _ in range(3):
        fs.step(1, 1)
        o.step()
    g = fs.fetch()
    assert np.array_equal(g["nthro"], o.nthro)
    np.testing.assert_allclose(g["pos"], o.pos, atol=1e-5)
    _close_rel(g["vel"], o.vel, 1e-4)
    np.testing.assert_allclose(g["Area64"], o.area, rtol=1e-5)
    np.testing.assert_allclose(g["Vol64"], o.vol, rtol=1e-5)


def test_fused_aggregation(cuda_device):
    from gpucell_gb300.fused import FusedSystem
    phys = gen.Physics(sur_energy=5.0, max_cut=1.2, zero_len=0.3, sca_fac=4.0)
    cfg = gen.channel(nx=24, ny=12, nz=18, wall_layers=3, b1_layers=1, cell_subdiv=2, cell_diameter=3.0,
                      phys=phys, cell_centers=[(0.0, -0.55, 0.0), (0.0, 0.55, 0.0)], seed=11, name="two_cells")
    fs = FusedSystem(cfg, noise=False)
    o = _oracle(cfg, False)
    for _ in range(2):
        fs.step(1, 1)
        o.step()
    g = fs.fetch()
    assert np.abs(o.aggforce).max() > 0
    _close_rel(g["AggForce"], o.aggforce, 2e-5)
    # Near rest the deformation force is a small net of large area/volume
    # terms (k (A - A0)/A0 dA/dx with k = 5000): compare on the scale of one
    # term, k times a mean edge length, not on the scale of the net.
    edge = float(np.mean(o.refedgelen))
    np.testing.assert_allclose(g["DefForce"], o.defforce, atol=1e-5 * phys.hgarea * edge)
    np.testing.assert_allclose(g["pos"], o.pos, atol=1e-5)


def test_fused_store_load_round_trip(cuda_device):
    from gpucell_gb300.fused import FusedSystem
    cfg = gen.small_channel()
    fs = FusedSystem(cfg, noise=True)
    fs.step(2, 1)
    a = fs.fetch()
    fs.load(a["pos"], a["vel"], a["velhalf"], a["force"], a["nthro"])
    b = fs.fetch()
    for k in ("pos", "vel", "velhalf", "force", "nthro"):
        assert np.array_equal(a[k], b[k]), k
    fs.step(1, 1)      # continues from the reloaded state
    assert np.isfinite(fs.fetch()["pos"]).all()


def test_fused_tracks_oracle_noise_on(cuda_device):
    """With the thermal noise on: the GPU and the oracle draw the same
    Philox pair noise (same key schedule, same 21-bit variates), so the
    trajectories agree to FP32 rounding: positions within 1e-5 and
    velocities within 1e-4 of their largest magnitude after 4 steps."""
    from gpucell_gb300.fused import FusedSystem
    cfg = gen.small_channel()
    fs = FusedSystem(cfg, noise=True)
    o = _oracle(cfg, True)
    for _ in range(4):
        o.step()
    fs.step(4, 1)
    g = fs.fetch()
    assert np.isfinite(o.vel).all()
    assert np.abs(o.vel).max() > 0.1     # the noise acts
    np.testing.assert_allclose(g["pos"], o.pos, atol=1e-5)
    _close_rel(g["vel"], o.vel, 1e-4)
    np.testing.assert_allclose(g["Area64"], o.area, rtol=1e-5)


def test_fused_force_evaluation_matches_oracle(cuda_device):
    """Forces of the fused step and of the FP64 oracle on the same positions
    (a vanishing time step leaves the set-up state in place; noise off), on
    a periodic suspension whose cells cross the box faces: per particle
    |dF_i| <= 1e-5 |F_i| + 16 u S_i (u FP32's unit roundoff, S_i the sum of
    the magnitudes of the terms F_i adds up, the pressure counted at c^2 rho
    since it amplifies the density's rounding); against the oracle's forces
    from the GPU's own densities and pressures, the same bound with the pressure counted at
    |P|; and the membrane deformation force
    of the undeformed cells, exactly zero, below 1e-3 (measured 1.1e-4; the
    edge and triangle vectors are differences of double-float positions, so
    a cell's geometry is the same wrapped into the box or not — with FP32
    differences it was 3.2e-3)."""
    import dataclasses
    from gpucell_gb300.fused import FusedSystem
    cfg = gen.suspension(nx=40, ny=40, nz=40, ncells=3, subdiv=3, seed=5)
    cfg = dataclasses.replace(cfg, phys=dataclasses.replace(cfg.phys, dt=1e-20))
    lo, hi = cfg.bbox[0::2], cfg.bbox[1::2]
    m = cfg.coor[cfg.n_cell_start:]
    assert ((m < lo) | (m >= hi)).any(), "no membrane vertex outside the box"
    o = _oracle(cfg, noise=False)
    o.step()
    fs = FusedSystem(cfg, noise=False)
    fs.step(1, 1)
    g = fs.fetch()
    fs.close()
    mov = slice(cfg.n_b1 + cfg.n_b2, cfg.n)
    from oracle.binding import force_error_stats
    s = force_error_stats(g["force"][mov], o.force[mov], o.force_scale()[mov], rtol=1e-5)
    # the same forces re-evaluated by the oracle from the GPU's FP32 densities and pressures:
    # the pressure's amplification of the density rounding drops out
    o.forces_from_density(g["rho"], g["press"])
    t = force_error_stats(g["force"][mov], o.force[mov], o.force_scale(31)[mov], rtol=1e-5)
    for name, x in (("own density", s), ("GPU density", t)):
        print(f"\nforce ({name}): median rel {x['median_rel']:.2e}, p99 {x['p99_rel']:.2e}, max {x['max_rel']:.2e}, "
              f"{100 * x['frac_within_rtol']:.2f} % within 1e-5, worst/bound {x['worst_ratio']:.2f} {x['worst']}")
    print(f"|DefForce| at rest {np.abs(g['DefForce']).max():.2e}")
    assert s["worst_ratio"] <= 1.0 and t["worst_ratio"] <= 1.0
    assert np.abs(g["DefForce"]).max() < 1e-3


@pytest.mark.parametrize("graph", [False, True])
def test_lists_grow_when_they_overflow(cuda_device, graph):
    """A handle created with room for 16 list entries per particle (the
    lists need ~140) grows its lists when a build overflows them and steps
    exactly as a handle with the default capacity: only the stride of the
    interleaved lists differs, not their entries or their order."""
    from gpucell_gb300.fused import FusedSystem
    cfg = gen.suspension(nx=24, ny=24, nz=24, ncells=1, subdiv=2, hematocrit=0.1, seed=3)
    small = FusedSystem(cfg, noise=True, list_capacity=16, graph=graph)
    ref = FusedSystem(cfg, noise=True, graph=graph)
    small.step(30, 1)
    ref.step(30, 1)
    a, b = small.fetch(), ref.fetch()
    assert small.stats()["capacity"] >= small.stats()["max_neighbors"] > 16
    assert small.flags() == 0 and ref.flags() == 0
    for k in ("pos", "vel", "force", "rho"):
        assert np.array_equal(a[k], b[k]), k
    small.close()
    ref.close()


def test_load_positions_several_boxes_away(cuda_device):
    """Positions loaded three box lengths off along each periodic axis (with
    crossing counts three lower, the same unwrapped state) step like the
    wrapped ones: the permutation wraps any number of lengths and counts them."""
    from gpucell_gb300.fused import FusedSystem
    cfg = gen.suspension(nx=24, ny=24, nz=24, ncells=1, subdiv=2, hematocrit=0.1, seed=3)
    a = FusedSystem(cfg, noise=False)
    a.step(5, 1)
    s = a.fetch()
    L = (cfg.bbox[1::2] - cfg.bbox[0::2]).astype(np.float32)
    far = FusedSystem(cfg, noise=False)
    far.load(s["pos"] + 3.0 * L, vel=s["vel"], velhalf=s["velhalf"], force=s["force"], nthro=s["nthro"] - 3)
    near = FusedSystem(cfg, noise=False)
    near.load(s["pos"], vel=s["vel"], velhalf=s["velhalf"], force=s["force"], nthro=s["nthro"])
    far.step(5, 1)
    near.step(5, 1)
    g, h = far.fetch(), near.fetch()
    assert far.flags() == 0 and near.flags() == 0
    assert np.array_equal(g["nthro"], h["nthro"])
    np.testing.assert_allclose(g["pos"], h["pos"], atol=2e-5)
    np.testing.assert_allclose(g["vel"], h["vel"], atol=2e-3 * np.abs(h["vel"]).max())
    for fs in (a, far, near):
        fs.close()


def test_device_buffers_load_and_store_like_host_ones(cuda_device):
    """gc_fused_store/store_cells/load with device pointers (to_device /
    from_device = 1, no staging) give the arrays the host path gives, and a
    state loaded from device buffers steps like the same state loaded from
    the host."""
    import ctypes as C
    import torch
    from gpucell_gb300 import _lib
    from gpucell_gb300.fused import FusedSystem
    cfg = gen.small_channel()
    fs = FusedSystem(cfg, noise=True)
    fs.step(3, 1)
    host = fs.fetch()
    n, dev = cfg.n, torch.device("cuda:0")
    d = {k: torch.empty((n, 3), dtype=torch.float32, device=dev) for k in ("pos", "vel", "force", "velhalf")}
    d["rho"], d["press"] = torch.empty(n, device=dev), torch.empty(n, device=dev)
    d["nthro"] = torch.empty((n, 3), dtype=torch.int32, device=dev)
    p = lambda t: C.c_void_p(t.data_ptr())
    _lib.call("gc_fused_store", fs.h, *[p(d[k]) for k in ("pos", "vel", "rho", "press", "force", "velhalf", "nthro")], 1)
    torch.cuda.synchronize()
    for k in ("pos", "vel", "rho", "press", "force", "velhalf", "nthro"):
        assert np.array_equal(d[k].cpu().numpy(), host[k]), k
    cells = {k: torch.empty(v.shape, dtype=torch.float32, device=dev)
             for k, v in host.items() if k in ("Area", "Vol", "DefForce", "AggForce", "TriNorDir", "TriCenter", "ParArea")}
    _lib.call("gc_fused_store_cells", fs.h, *[p(cells[k]) for k in ("Area", "Vol", "DefForce", "AggForce",
                                                                     "TriNorDir", "TriCenter", "ParArea")], 1)
    torch.cuda.synchronize()
    for k, t in cells.items():
        assert np.array_equal(t.cpu().numpy(), host[k]), k
    fs.step(2, 1)                    # move on, then load the stored state back from the device buffers
    _lib.call("gc_fused_load", fs.h, *[p(d[k]) for k in ("pos", "vel", "velhalf", "force", "nthro")], 1)
    fs.step(4, 1)
    got = fs.fetch()
    ref = FusedSystem(cfg, noise=True)
    ref.step(5, 1)                   # the same step indices key the same noise
    ref.load(host["pos"], host["vel"], host["velhalf"], host["force"], host["nthro"])
    ref.step(4, 1)
    want = ref.fetch()
    for k in ("pos", "vel", "force"):
        assert np.array_equal(got[k], want[k]), k
    fs.close()
    ref.close()


@pytest.mark.parametrize("graph", [False, True])
def test_step_store_matches_step_then_store(cuda_device, graph):
    """gc_fused_step_store (the outputs that are final early in the step
    copied beside the rest of it) returns exactly what a step followed by
    gc_fused_store and gc_fused_store_cells returns, across list rebuilds:
    a walled channel with a cell, and a Couette rouleau with Morse
    aggregation."""
    from gpucell_gb300.fused import FusedSystem
    phys = gen.Physics(sur_energy=5.0, max_cut=1.2, zero_len=0.3, sca_fac=4.0)
    cfgs = [gen.small_channel(),
            gen.couette(nx=36, ny=18, nz=24, ncells=2, subdiv=2, cell_diameter=3.0, shear_rate=0.5, seed=31,
                        phys=phys)]
    for cfg in cfgs:
        a = FusedSystem(cfg, noise=True, skin=0.03, graph=graph)
        b = FusedSystem(cfg, noise=True, skin=0.03, graph=graph)
        for _ in range(12):
            got = a.step_fetch(1)
            b.step(1, 1)
            want = b.fetch()
            for k, v in got.items():
                assert np.array_equal(v, want[k]), k
        assert a.stats()["rebuilds"] >= 2 and a.flags() == 0
        a.close()
        b.close()
