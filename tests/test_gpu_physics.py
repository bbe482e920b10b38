"""Physics of the fused step against the FP64 oracle and against theory.

* equipartition: with the pair noise on, a periodic fluid box thermalises
  to m <v^2>/3 = kT within 3 % (measured 0.75 %), with Gaussian-like
  velocity components (kurtosis 3 +- 0.3) and no net momentum;
* Poiseuille flow between Bound2 walls (noise off): after 300 steps from
  the analytic start the binned velocity profile is within 1e-4 u_max of the
  oracle's (measured 1.4e-7) and within 5 % u_max of the analytic parabola
  (measured 2.8 %: the SPH discretisation of the viscous term);
* membrane area and volume follow the oracle within 1e-5 relative over 300
  steps (measured 1.1e-7);
* trajectory drift against the oracle over 1000 steps (noise off) stays
  below 5e-5 cut-off radii (measured 5.3e-6);
* double-float positions: particles far from the origin under a small body
  force stay within one FP32 ulp of the FP64 oracle over 1000 steps, where
  plain FP32 accumulation of the same displacements loses most of them.
"""
import numpy as np
import pytest

from gpucell_gb300 import generator as gen

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def _oracle(cfg, noise):
    from oracle.binding import Oracle
    o = Oracle(cfg, noise=noise)
    o.setup()
    return o


def test_equipartition_and_momentum(cuda_device):
    from gpucell_gb300.fused import FusedSystem
    cfg = gen.suspension(nx=24, ny=24, nz=24, ncells=0, seed=5)
    kT, m = cfg.phys.temp, cfg.phys.mass
    fs = FusedSystem(cfg, noise=True)
    fs.step(300, 0)
    temps, kurt, pmean = [], [], []
    for _ in range(15):
        fs.step(20, 0)
        v = fs.fetch()["vel"].astype(np.float64)
        temps.append(m * (v * v).sum(axis=1).mean() / 3.0)
        c = v - v.mean(axis=0)
        kurt.append(((c ** 4).mean(axis=0) / (c ** 2).mean(axis=0) ** 2).mean())
        pmean.append(np.abs(v.mean(axis=0)).max() / np.sqrt(kT / m))
    T = float(np.mean(temps))
    print(f"\nequipartition: T/kT = {T / kT:.4f}, kurtosis = {np.mean(kurt):.3f}, max |<v>|/v_th = {max(pmean):.2e}")
    assert abs(T / kT - 1.0) < 0.03
    assert 2.7 < np.mean(kurt) < 3.3
    assert max(pmean) < 0.01
    assert fs.flags() == 0


def _poiseuille_cfg():
    phys = gen.Physics(shear_vis=50.0, ext_force=1.0, sound1=20.0)
    return gen.channel(nx=24, ny=12, nz=12, wall_layers=3, b1_layers=0, cell_subdiv=-1, phys=phys, seed=21,
                       name="poiseuille")


def _profile(pos, vel, cfg, nbins=8):
    fl = slice(cfg.n_b1 + cfg.n_b2, cfg.n_cell_start)
    y, u = pos[fl, 1], vel[fl, 0]
    lo, hi = float(cfg.bbox[2]), float(cfg.bbox[3])
    b = np.clip(((y - lo) / (hi - lo) * nbins).astype(int), 0, nbins - 1)
    prof = np.array([u[b == k].mean() for k in range(nbins)])
    yc = lo + (np.arange(nbins) + 0.5) * (hi - lo) / nbins
    return yc, prof


def test_poiseuille_profile(cuda_device):
    from gpucell_gb300.fused import FusedSystem
    cfg = _poiseuille_cfg()
    rho, g, eta = cfg.den_init, cfg.phys.ext_force, cfg.phys.shear_vis
    h = 0.5 * float(cfg.bbox[3] - cfg.bbox[2])
    umax = rho * g * h * h / (2 * eta)
    pos = cfg.coor.astype(np.float64)
    vel = np.zeros((cfg.n, 3))
    fl = slice(cfg.n_b1 + cfg.n_b2, cfg.n_cell_start)
    vel[fl, 0] = rho * g / (2 * eta) * (h * h - pos[fl, 1] ** 2)
    vel = vel.astype(np.float32)
    fs = FusedSystem(cfg, noise=False)
    fs.load(cfg.coor, vel)
    o = _oracle(cfg, False)
    o.set(vel=vel.astype(np.float64))
    for _ in range(300):
        o.step()
    fs.step(300, 1)
    g_ = fs.fetch()
    yc, pg = _profile(g_["pos"], g_["vel"], cfg)
    _, po = _profile(o.pos, o.vel, cfg)
    ua = rho * g / (2 * eta) * (h * h - yc ** 2)
    err_oracle = np.abs(pg - po).max() / umax
    err_analytic = np.abs(pg - ua).max() / umax
    print(f"\npoiseuille: u_max {umax:.4f}, GPU vs oracle {err_oracle:.2e}, GPU vs analytic {err_analytic:.3f}")
    assert err_oracle < 1e-4
    assert err_analytic < 0.05


def test_cell_area_volume_track_oracle(cuda_device):
    from gpucell_gb300.fused import FusedSystem
    cfg = gen.small_channel()
    fs = FusedSystem(cfg, noise=False)
    o = _oracle(cfg, False)
    worst_a = worst_v = 0.0
    for _ in range(6):
        fs.step(50, 1)
        for _ in range(50):
            o.step()
        g = fs.fetch()
        worst_a = max(worst_a, abs(g["Area64"][0] / o.area[0] - 1))
        worst_v = max(worst_v, abs(g["Vol64"][0] / o.vol[0] - 1))
    print(f"\ncell: max relative area error {worst_a:.2e}, volume error {worst_v:.2e} over 300 steps")
    assert worst_a < 1e-5 and worst_v < 1e-5


def test_trajectory_drift_1000_steps(cuda_device):
    from gpucell_gb300.fused import FusedSystem
    cfg = gen.small_channel()
    fs = FusedSystem(cfg, noise=False)
    o = _oracle(cfg, False)
    drift = []
    for _ in range(10):
        fs.step(100, 1)
        for _ in range(100):
            o.step()
        g = fs.fetch()
        d = g["pos"].astype(np.float64) - o.pos
        L = float(cfg.bbox[1] - cfg.bbox[0])
        d[:, 0] -= L * np.rint(d[:, 0] / L)
        Lz = float(cfg.bbox[5] - cfg.bbox[4])
        d[:, 2] -= Lz * np.rint(d[:, 2] / Lz)
        drift.append(np.abs(d).max())
    print("\ndrift per 100 steps: " + " ".join(f"{x:.1e}" for x in drift))
    assert drift[-1] < 5e-5


def test_gpu_diagnostics_match_the_stored_state(cuda_device):
    """gc_ensemble_diagnostics (FP64 on the GPU) equals the same sums taken
    in FP64 on the host from the stored state, and the momentum of a
    periodic fluid without body force stays at zero."""
    from gpucell_gb300.fused import FusedSystem
    cfg = gen.suspension(nx=24, ny=24, nz=24, ncells=0, seed=5)
    fs = FusedSystem(cfg, noise=True)
    fs.step(50, 1)
    g = fs.fetch()
    d = fs.diagnostics()
    m = cfg.phys.mass
    v = g["vel"].astype(np.float64)[cfg.n_b1 + cfg.n_b2:]
    P = m * v.sum(axis=0)
    E = 0.5 * m * (v * v).sum()
    T = (2 * E - (P * P).sum() / (m * v.shape[0])) / (3 * v.shape[0])
    np.testing.assert_allclose(d["momentum"], P, rtol=1e-9, atol=1e-9)
    assert abs(d["kinetic_energy"] / E - 1) < 1e-12 and abs(d["temperature"] / T - 1) < 1e-12
    assert d["max_speed"] == pytest.approx(np.sqrt((v * v).sum(axis=1)).max(), rel=1e-12)
    rho = g["rho"].astype(np.float64)[cfg.n_b1 + cfg.n_b2:cfg.n_cell_start]
    assert d["mean_fluid_density"] == pytest.approx(rho.mean(), rel=1e-6)
    assert d["moving"] == v.shape[0]
    assert np.abs(d["momentum"]).max() < 1e-6 * np.sqrt(2 * E * m * v.shape[0])   # pairwise forces, no drive


def _sparse_gas(x0=100.0, spacing=1.5, nx=64, nyz=4, g=0.02):
    """Fluid particles farther apart than the cut-off (no pairs act), at
    x in [x0, x0 + nx*spacing), in a periodic box; only the body force
    moves them."""
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(nyz), np.arange(nyz), indexing="ij")
    coor = np.stack([x0 + spacing * ix, spacing * (iy + 0.5), spacing * (iz + 0.5)], -1).reshape(-1, 3)
    coor = coor.astype(np.float32)
    L = spacing * nyz
    return gen.Config(name="sparse_gas", bbox=np.array([0, 2 * x0, 0, L, 0, L], np.float32), pmask=7, n_b1=0,
                      n_b2=0, n_fluid=coor.shape[0], coor=coor, velhalf=np.zeros_like(coor),
                      den_init=gen.lattice_density(1.0 / 3.0), phys=gen.Physics(ext_force=g))


def test_double_float_positions_far_from_the_origin(cuda_device):
    """At x ~ 100-200 an FP32 ulp is 7.6e-6-1.5e-5, larger than the per-step
    displacement dt*v (< 2e-8 * step for g = 0.02, dt = 1e-3): FP32 positions
    do not move for hundreds of steps.  The fused step keeps each position as
    an FP32 value plus its FP32 remainder and must track the FP64 oracle to
    within one ulp of the stored FP32 value."""
    from gpucell_gb300.fused import FusedSystem
    cfg = _sparse_gas()
    fs = FusedSystem(cfg, noise=False)
    fs.step(1000, 1)
    g = fs.fetch()
    o = _oracle(cfg, False)
    for _ in range(1000):
        o.step()
    x_gpu = g["pos"].astype(np.float64)
    ulp = np.spacing(np.abs(g["pos"])).astype(np.float64)
    err = np.abs(x_gpu - o.pos)
    moved = o.pos[:, 0] - cfg.coor[:, 0].astype(np.float64)
    # the same displacements accumulated in FP32, for the record
    x32 = cfg.coor[:, 0].copy()
    v = np.zeros_like(x32)
    dt, a = np.float32(cfg.phys.dt), np.float32(cfg.phys.ext_force)
    h, lam = np.float32(0.5) * dt * dt, np.float32(0.5) * dt
    f = np.zeros_like(x32)
    for _ in range(1000):
        x32 = x32 + (dt * v + h * f)
        f_new = np.full_like(x32, a)
        v = v + lam * (f + f_new)
        f = f_new
    err32 = np.abs(x32.astype(np.float64) - o.pos[:, 0])
    print(f"\ndisplacement {moved.mean():.3e}; |GPU - oracle| max {err.max():.2e} "
          f"({(err / ulp).max():.2f} ulp); FP32 accumulation would be off by {err32.max():.2e} "
          f"({(err32 / ulp[:, 0]).max():.0f} ulp)")
    assert moved.min() > 5e-3
    assert (err <= ulp).all()
