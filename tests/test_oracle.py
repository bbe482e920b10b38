"""The FP64 oracle against analytic known answers, finite differences of its
own energies, and conservation laws (no GPU)."""
import json
import math
import os

import numpy as np
import pytest

from gpucell_gb300 import generator as gen

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "analytic.json")))


def _pair_config(x0, x1, pmask=0, box=10.0):
    """Two fluid particles in a closed box (no walls, no cells)."""
    coor = np.array([x0, x1], np.float32)
    cfg = gen._assemble("pair", [-box, box, -box, box, -box, box], pmask, np.zeros((0, 3)), np.zeros((0, 3)), coor,
                        [], gen.Physics(), 1.0 / 3.0)
    return cfg


def test_philox_matches_independent_python(oracle_lib):
    from oracle.binding import noise_key, philox, philox2
    for case in GOLDEN["philox"]:
        assert philox(case["ctr"], case["key"]) == case["out"]
    for case in GOLDEN["philox2"]:
        assert philox2(case["ctr"], case["key"]) == case["out"]
    for case in GOLDEN["noise_key"]:
        assert noise_key(case["seed"], case["step"]) == case["key"]


def test_pair_noise_moments_and_antisymmetry(oracle_lib):
    """xi_ij = -xi_ji; over many pairs the components have zero mean, unit
    variance and no correlation (uniform on [-sqrt 3, sqrt 3])."""
    from oracle.binding import Oracle
    cfg = _pair_config([0.0, 0.0, 0.0], [0.3, 0.0, 0.0])
    o = Oracle(cfg, noise=True)
    rng = np.random.default_rng(0)
    ids = rng.integers(0, 1 << 22, size=(20000, 2))
    xs = np.array([o.pair_noise(int(a), int(b)) for a, b in ids if a != b])
    np.testing.assert_allclose(o.pair_noise(5, 9), -o.pair_noise(9, 5))
    assert abs(xs.mean()) < 0.02 and abs(xs.var() - 1.0) < 0.03
    cc = np.corrcoef(xs.T)
    assert np.abs(cc - np.eye(3)).max() < 0.03
    assert xs.max() <= 3 ** 0.5 and xs.min() >= -(3 ** 0.5)


def test_wendland_values_and_normalisation(oracle_lib):
    from oracle.binding import Oracle
    for case in GOLDEN["wendland"]:
        r = case["r"]
        if r == 0.0:
            continue
        cfg = _pair_config([0.0, 0.0, 0.0], [r, 0.0, 0.0])
        o = Oracle(cfg, noise=False)
        o.call("density")
        np.testing.assert_allclose(o.rho[0], GOLDEN["wendland"][0]["W"] + case["W"], rtol=1e-6)
    # integral of W over the support is 1
    r = np.linspace(0.0, 1.0, 200001)
    s = r
    W = 21.0 / (2.0 * math.pi) * (1 - s) ** 4 * (1 + 4 * s)
    assert abs(np.trapezoid(4 * math.pi * r * r * W, r) - 1.0) < 1e-8


def test_sdpd_pair_force_against_hand_formula(oracle_lib):
    from oracle.binding import Oracle
    for case in GOLDEN["sdpd_pair"]:
        cfg = _pair_config(case["xi"], case["xj"])
        cfg.phys.shear_vis, cfg.phys.bulk_vis = case["eta"], case["zeta"]
        o = Oracle(cfg, noise=False)
        # positions enter as float32, as on the GPU
        xi = np.float32(case["xi"]).astype(float)
        xj = np.float32(case["xj"]).astype(float)
        o.set(vel=np.array([case["vi"], case["vj"]]), rho=np.array([case["rho_i"], case["rho_j"]]),
              press=np.array([case["P_i"], case["P_j"]]))
        o.call("sdpd_force")
        want = np.array(case["force_i"])
        # the fixture used the unrounded positions; allow for the float32 rounding
        tol = 1e-5 * np.abs(want).max() + 1e-6
        np.testing.assert_allclose(o.force[0], want, atol=tol)
        np.testing.assert_allclose(o.force[1], -o.force[0], atol=1e-12)   # Newton's third law
        del xi, xj


def _ico_config(scale=1.0, subdiv=0, shear=100.0):
    v, f = gen.icosphere(subdiv)
    phys = gen.Physics(shear_mod=shear)
    return gen._assemble("ico", [-20, 20, -20, 20, -20, 20], 0, np.zeros((0, 3)), np.zeros((0, 3)), np.zeros((0, 3)),
                         [(v * scale, f)], phys, 1.0 / 3.0), phys


def test_icosahedron_geometry(oracle_lib):
    from oracle.binding import Oracle
    cfg, _ = _ico_config()
    o = Oracle(cfg, noise=False)
    o.setup()
    g = GOLDEN["icosahedron"]
    np.testing.assert_allclose(o.area[0], g["area"], rtol=1e-6)
    np.testing.assert_allclose(o.vol[0], g["volume"], rtol=1e-6)
    np.testing.assert_allclose(np.abs(o.refangle), g["dihedral"], rtol=1e-6)
    np.testing.assert_allclose(o.refedgelen, g["edge"], rtol=1e-6)
    np.testing.assert_allclose(o.pararea.sum(), o.area[0], rtol=1e-12)
    # outward normals: centroid . normal > 0 on a sphere
    assert (np.einsum("ij,ij->i", o.tricenter, o.trinormal) > 0).all()


def test_wlc_pow_constants_and_zero_force_at_rest(oracle_lib):
    from oracle.binding import Oracle
    case = GOLDEN["wlc_pow"][0]
    edge = GOLDEN["icosahedron"]["edge"]
    cfg, phys = _ico_config(scale=case["l0"] / edge, shear=case["mu0"])
    o = Oracle(cfg, noise=False)
    o.setup()
    np.testing.assert_allclose(o.perlen, case["p"], rtol=1e-5)
    np.testing.assert_allclose(o.hpow, case["kp"], rtol=1e-5)
    np.testing.assert_allclose(o.maxrefedgelen, case["lmax"], rtol=1e-5)
    o.call("geo", 0)
    o.call("def_force")
    assert np.abs(o.defforce).max() < 1e-6 * case["mu0"]


@pytest.mark.parametrize("seed", [0, 1])
def test_membrane_force_is_energy_gradient(oracle_lib, seed):
    from oracle.binding import Oracle
    cfg = gen.small_channel()
    o = Oracle(cfg, noise=False)
    o.setup()
    rng = np.random.default_rng(seed)
    ncs = cfg.n_cell_start
    o.pos[ncs:] += rng.normal(scale=0.02, size=o.pos[ncs:].shape)
    o.call("geo", 0)
    o.force[:] = 0
    o.call("def_force")
    F = o.force[ncs:].copy()
    h = 1e-6
    for v in rng.choice(cfg.ncp, 8, replace=False):
        for a in range(3):
            o.pos[ncs + v, a] += h
            ep = o.membrane_energy()
            o.pos[ncs + v, a] -= 2 * h
            em = o.membrane_energy()
            o.pos[ncs + v, a] += h
            assert abs(F[v, a] + (ep - em) / (2 * h)) < 1e-6 * (1.0 + np.abs(F).max())


def test_morse_force_is_energy_gradient(oracle_lib):
    from oracle.binding import Oracle
    v, f = gen.icosphere(1)
    shape = gen.biconcave(v, 2.0)
    phys = gen.Physics(sur_energy=3.0, max_cut=0.8, zero_len=0.3, sca_fac=4.0)
    cells = [(shape, f), (shape + np.array([0.0, 0.0, 0.95]), f)]
    cfg = gen._assemble("two", [-10, 10, -10, 10, -10, 10], 0, np.zeros((0, 3)), np.zeros((0, 3)), np.zeros((0, 3)),
                        cells, phys, 1.0 / 3.0)
    o = Oracle(cfg, noise=False)
    o.setup()
    o.force[:] = 0
    o.call("agg_force")
    assert np.abs(o.aggforce).max() > 0
    np.testing.assert_allclose(o.aggforce.sum(axis=0), 0.0, atol=1e-9)
    rng = np.random.default_rng(3)
    h = 1e-6
    moved = np.nonzero(np.abs(o.aggforce).sum(1) > 0)[0]
    for vtx in rng.choice(moved, min(6, moved.size), replace=False):
        for a in range(3):
            o.pos[vtx, a] += h
            ep = o.morse_energy()
            o.pos[vtx, a] -= 2 * h
            em = o.morse_energy()
            o.pos[vtx, a] += h
            fd = -(ep - em) / (2 * h)
            assert abs(o.aggforce[vtx, a] - fd) < 1e-5 * (1.0 + abs(fd)), (vtx, a)


def test_sdpd_conserves_momentum_with_noise(oracle_lib):
    from oracle.binding import Oracle
    cfg = gen.suspension(nx=12, ny=12, nz=12, ncells=0)
    o = Oracle(cfg, noise=True)
    rng = np.random.default_rng(5)
    o.set(vel=rng.normal(size=(cfg.n, 3)))
    o.call("density")
    o.call("eos")
    o.call("sdpd_force")
    tot = o.force.sum(axis=0)
    assert np.abs(tot).max() < 1e-9 * np.abs(o.force).sum()


def test_neighbor_stats_match_brute_force(oracle_lib):
    from oracle.binding import Oracle
    cfg = gen.small_channel()
    o = Oracle(cfg, noise=False)
    cnt, h = o.neighbor_stats()
    x = cfg.coor.astype(np.float32)
    L = np.float32(cfg.bbox[1]) - np.float32(cfg.bbox[0])
    Lz = np.float32(cfg.bbox[5]) - np.float32(cfg.bbox[4])
    for i in np.random.default_rng(0).choice(cfg.n, 64, replace=False):
        d = x[i] - x
        for a, LL in ((0, L), (2, Lz)):
            half = np.float32(0.5) * LL
            d[:, a] = np.where(d[:, a] > half, d[:, a] - LL, np.where(d[:, a] < -half, d[:, a] + LL, d[:, a]))
        r2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        nb = np.nonzero(r2 < np.float32(1.0))[0]
        nb = nb[nb != i]
        assert cnt[i] == nb.size


def test_full_step_is_stable(oracle_lib):
    """20 steps of the channel with a cell stay finite and keep the cell's
    area and volume within 10% (the membrane starts inside the fluid
    lattice, so the pressure transient moves it)."""
    from oracle.binding import Oracle
    cfg = gen.small_channel()
    o = Oracle(cfg, noise=False)
    o.setup()
    a0, v0 = o.area.copy(), o.vol.copy()
    for _ in range(20):
        o.step()
    assert np.all(np.isfinite(o.pos)) and np.all(np.isfinite(o.vel))
    assert abs(o.area[0] / a0[0] - 1) < 0.1 and abs(o.vol[0] / v0[0] - 1) < 0.1


def test_noise_on_steps_stay_finite_and_hot():
    """Regression: a pair that passes the FP32 cut-off test while its FP64
    distance is a rounding error above rc gets a tiny negative F; its noise
    amplitude must be zero, not sqrt of a negative number (which turned the
    whole state into NaN within a few steps)."""
    import os
    from oracle.binding import Oracle
    from gpucell_gb300 import generator as gen
    cfg = gen.suspension(nx=24, ny=16, nz=16, ncells=0, seed=12345)
    o = Oracle(cfg, noise=True, nthreads=os.cpu_count() or 1)
    o.setup()
    for _ in range(6):
        o.step()
        assert np.isfinite(o.pos).all() and np.isfinite(o.vel).all() and np.isfinite(o.force).all()
    assert (o.vel ** 2).sum(axis=1).mean() > 0.1   # the noise heats the fluid


@pytest.mark.parametrize("noise", [False, True])
def test_force_scale_bounds_every_force(oracle_lib, noise):
    """The per-particle scale of the force comparisons (the sum of the
    magnitudes of the terms a force adds up) is at least the force itself,
    part by part and in total (triangle inequality), on a walled channel
    with a cell and on a periodic suspension with Morse aggregation."""
    import dataclasses
    from oracle.binding import Oracle
    phys = dataclasses.replace(gen.Physics(), sur_energy=5.0, max_cut=1.2, zero_len=0.3, sca_fac=4.0)
    for cfg in (gen.small_channel(), gen.suspension(nx=24, ny=24, nz=24, ncells=2, subdiv=2, hematocrit=0.15,
                                                    seed=3, phys=phys)):
        o = Oracle(cfg, noise=noise)
        o.setup()
        o.step()
        o.step()
        f = np.linalg.norm(o.force, axis=1)
        s = o.force_scale()
        mov = np.arange(cfg.n) >= cfg.n_b1 + cfg.n_b2
        assert (s[mov] >= f[mov] * (1 - 1e-12)).all()
        assert (s[~mov] == 0).all()
        cs = cfg.n_cell_start
        sm = o.force_scale(o.SCALE_MEMB)[cs:]
        assert (sm >= np.linalg.norm(o.defforce, axis=1) * (1 - 1e-12)).all()
        if cfg.phys.sur_energy:
            sa = o.force_scale(o.SCALE_MORSE)[cs:]
            assert (sa >= np.linalg.norm(o.aggforce, axis=1) * (1 - 1e-12)).all()
        assert np.allclose(s, sum(o.force_scale(p) for p in (1 | 32, 2, 4, 8, 16)))
        assert (o.force_scale(31) <= s).all()
