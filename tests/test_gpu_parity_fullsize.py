"""The fused step against the FP64 oracle at the benchmark's own sizes (the
step checked is Particle::UpdatePar, src/Particle.cu:1310-1329).

* The 4.2M-particle suspension (256 x 128 x 128 sites, 200 cells of 2562
  vertices, periodic):
  - one force evaluation on identical positions (a vanishing time step
    leaves the set-up state in place; noise off, because the random force
    scales as dt^-1/2): per particle |dF_i| <= 1e-5 |F_i| + 16 u S_i, with u
    FP32's unit roundoff and S_i the sum of the magnitudes of the terms F_i
    adds up (SDPD pair terms, membrane terms; from the oracle) -- 1e-5
    relative unless the net force cancels much larger terms.  The pressure
    P = c^2 (rho - rho0) turns the FP32 rounding of the density sum into an
    error of size c^2 rho u, so against the oracle's own densities its term
    counts at that size; against the oracle's forces from the GPU's
    densities and pressures, at |P|.  The median, 99th percentile and largest relative
    error |dF_i| / |F_i| and the fraction of particles within 1e-5 are
    printed for both.
  - five steps with the thermal noise on (both sides draw the same Philox
    pair noise): positions within 1e-5, velocities within 1e-4 of their
    largest magnitude, every cell's FP64 area and volume within 1e-6
    relative of the oracle's.
* The walled channel (64 x 32 x 32 fluid, 3 wall layers on each side, one
  642-vertex cell), 1000 steps from rest under the body force, noise off:
  the velocity profile across the channel (8 bins) within 1e-3 of its
  largest bin (the target is 1 %), positions within 1e-4 of the oracle's,
  the cell's area and volume within 1e-5 relative (the target is 1e-4).
"""
import dataclasses

import numpy as np
import pytest

from gpucell_gb300 import generator as gen

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


@pytest.fixture(scope="module")
def cfg2():
    return gen.suspension(seed=12345)


def _oracle(cfg, noise):
    import os
    from oracle.binding import Oracle
    o = Oracle(cfg, noise=noise, nthreads=os.cpu_count() or 1)
    o.setup()
    return o


def _min_image(d, cfg):
    d = d.copy()
    for a in range(3):
        if (cfg.pmask >> a) & 1:
            L = float(cfg.bbox[2 * a + 1] - cfg.bbox[2 * a])
            d[:, a] -= L * np.rint(d[:, a] / L)
    return d


def test_force_evaluation_at_full_size(cuda_device, cfg2):
    from gpucell_gb300.fused import FusedSystem
    from oracle.binding import force_error_stats
    cfg = dataclasses.replace(cfg2, phys=dataclasses.replace(cfg2.phys, dt=1e-20))
    o = _oracle(cfg, noise=False)
    o.step()
    scale = o.force_scale()
    fs = FusedSystem(cfg, noise=False)
    fs.step(1, 1)
    g = fs.fetch()
    fs.close()
    mov = slice(cfg.n_b1 + cfg.n_b2, cfg.n)
    cs = cfg.n_cell_start - (cfg.n_b1 + cfg.n_b2)
    res = {}
    for label, sc in (("own density", scale), ("GPU density", None)):
        if sc is None:
            o.forces_from_density(g["rho"], g["press"])
            sc = o.force_scale(31)
        f, w, sm = g["force"][mov], o.force[mov], sc[mov]
        res[label] = [(name, force_error_stats(f[sl], w[sl], sm[sl], rtol=1e-5))
                      for name, sl in (("all", slice(None)), ("fluid", slice(0, cs)), ("membrane", slice(cs, None)))]
    for label, rows in res.items():
        for name, x in rows:
            print(f"\ncfg2 force vs oracle ({label}), {name} ({x['particles']}): median rel {x['median_rel']:.2e}, "
                  f"p99 {x['p99_rel']:.2e}, max {x['max_rel']:.2e}, {100 * x['frac_within_rtol']:.3f} % within "
                  f"1e-5, worst/bound {x['worst_ratio']:.3f} {x['worst']}")
    for label, rows in res.items():
        for name, x in rows:
            assert x["worst_ratio"] <= 1.0, (label, name, x["worst"])
    assert res["own density"][0][1]["median_rel"] < 1e-5


def test_five_steps_with_noise_at_full_size(cuda_device, cfg2):
    from gpucell_gb300.fused import FusedSystem
    o = _oracle(cfg2, noise=True)
    fs = FusedSystem(cfg2, noise=True, skin=0.075)
    fs.step(5, 1)
    for _ in range(5):
        o.step()
    g = fs.fetch()
    fs.close()
    assert fs_flags_ok(g)
    dpos = np.abs(_min_image(g["pos"].astype(np.float64) - o.pos, cfg2)).max()
    vs = np.abs(o.vel).max()
    dvel = np.abs(g["vel"] - o.vel).max() / vs
    ea = np.abs(g["Area64"] / o.area - 1).max()
    ev = np.abs(g["Vol64"] / o.vol - 1).max()
    print(f"\ncfg2 after 5 noisy steps: max|dpos| {dpos:.2e}, max|dvel|/max|v| {dvel:.2e} (max|v| {vs:.3f}), "
          f"area {ea:.2e}, volume {ev:.2e}")
    assert vs > 0.1            # the noise acts
    assert dpos < 1e-5
    assert dvel < 1e-4
    assert ea < 1e-6 and ev < 1e-6


def fs_flags_ok(g):
    return all(np.isfinite(g[k]).all() for k in ("pos", "vel", "force"))


def test_walled_channel_1000_steps(cuda_device):
    from gpucell_gb300.fused import FusedSystem
    cfg = gen.channel()
    assert cfg.n_fluid == 65536 and cfg.n_b2 == 12288 and cfg.ncp == 642
    o = _oracle(cfg, noise=False)
    fs = FusedSystem(cfg, noise=False)
    fs.step(1000, 1)
    for _ in range(1000):
        o.step()
    g = fs.fetch()
    flags = fs.flags()
    fs.close()
    fl = slice(cfg.n_b1 + cfg.n_b2, cfg.n_cell_start)
    lo, hi = float(cfg.bbox[2]), float(cfg.bbox[3])

    def profile(pos, vel):
        b = np.clip(((pos[fl, 1] - lo) / (hi - lo) * 8).astype(int), 0, 7)
        return np.array([vel[fl, 0][b == k].mean() for k in range(8)])

    pg, po = profile(g["pos"].astype(np.float64), g["vel"].astype(np.float64)), profile(o.pos, o.vel)
    eprof = np.abs(pg - po).max() / np.abs(po).max()
    dpos = np.abs(_min_image(g["pos"].astype(np.float64) - o.pos, cfg)).max()
    ea, ev = abs(g["Area64"][0] / o.area[0] - 1), abs(g["Vol64"][0] / o.vol[0] - 1)
    print(f"\ncfg1 after 1000 steps: profile error {eprof:.2e} of the largest bin ({np.abs(po).max():.3e}), "
          f"max|dpos| {dpos:.2e}, area {ea:.2e}, volume {ev:.2e}")
    assert flags == 0
    assert np.abs(po).max() > 0
    assert eprof < 1e-3
    assert dpos < 1e-4
    assert ea < 1e-5 and ev < 1e-5
