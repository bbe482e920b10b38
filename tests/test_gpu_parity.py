"""Every boundary entry point on the GPU against the FP64 oracle.

Each test puts the same state into the CUDA library (through the C ABI, in
the reference's slot-ordered layout) and into the oracle (original order),
runs one entry point on both and compares.  Tolerances, stated per test:
  * neighbour sets: bit-exact (count and id checksum per particle);
  * sums of positive terms (density, areas, volumes): 2e-6 relative;
  * forces, per particle: |dF_i| <= 1e-5 |F_i| + 16 u S_i, with u FP32's unit
    roundoff and S_i the sum of the magnitudes of the terms F_i adds up (from
    the oracle): 1e-5 relative unless the net force cancels much larger
    terms, then a few FP32 roundings of those terms;
  * elementwise integrator stages: 1e-6 relative to the data's scale.
"""
import ctypes as C

import numpy as np
import pytest

from gpucell_gb300 import generator as gen

pytestmark = pytest.mark.gpu


def _state(cfg, seed=0, wall_vel=0.0):
    rng = np.random.default_rng(seed)
    n = cfg.n
    mob = np.arange(n) >= cfg.n_b1 + cfg.n_b2
    pos = cfg.coor.astype(np.float64).copy()
    pos[mob] += rng.uniform(-0.04, 0.04, size=(mob.sum(), 3))
    pos = pos.astype(np.float32).astype(np.float64)
    vel = rng.normal(size=(n, 3)).astype(np.float32).astype(np.float64)
    rho = (cfg.den_init * (1 + 0.02 * rng.normal(size=n))).astype(np.float32).astype(np.float64)
    force = (10 * rng.normal(size=(n, 3))).astype(np.float32).astype(np.float64)
    velhalf = (rng.normal(size=(n, 3))).astype(np.float32).astype(np.float64)
    velhalf[cfg.n_b1:cfg.n_b1 + cfg.n_b2] = wall_vel
    press = (100 * rng.normal(size=n)).astype(np.float32).astype(np.float64)
    return dict(pos=pos, vel=vel, rho=rho, force=force, velhalf=velhalf, press=press)


def _pair(cfg, noise=False, seed=0, wall_vel=0.0):
    from gpucell_gb300.host import ParticleSystem
    from oracle.binding import Oracle
    ps = ParticleSystem(cfg, noise=noise)
    o = Oracle(cfg, noise=noise)
    o.setup()
    st = _state(cfg, seed, wall_vel)
    ps.set_state(**st)
    ps.con_cube_list()
    o.set(**st)
    return ps, o


def _sync_oracle(ps, o):
    """Copies the GPU state (original order) into the oracle."""
    g = ps.fetch()
    o.set(pos=g["pos"], vel=g["vel"], rho=g["rho"], press=g["press"], force=g["force"], velhalf=g["velhalf"],
          nthro=g["nthro"])
    return g


def _force_close(got, want, scale, rtol=1e-5, what="force"):
    from oracle.binding import assert_forces_close
    s = assert_forces_close(got, want, scale, rtol=rtol, what=what)
    print(f"\n{what}: median rel {s['median_rel']:.2e}, p99 {s['p99_rel']:.2e}, max {s['max_rel']:.2e}, "
          f"{100 * s['frac_within_rtol']:.2f} % within {rtol:g}, worst/bound {s['worst_ratio']:.2f}")
    return s


@pytest.fixture(scope="module")
def channel_cfg():
    return gen.small_channel()


@pytest.fixture(scope="module")
def two_cell_cfg():
    phys = gen.Physics(sur_energy=5.0, max_cut=1.2, zero_len=0.3, sca_fac=4.0)
    return gen.channel(nx=24, ny=12, nz=18, wall_layers=3, b1_layers=1, cell_subdiv=2, cell_diameter=3.0,
                       phys=phys, cell_centers=[(0.0, -0.55, 0.0), (0.0, 0.55, 0.0)], seed=11, name="two_cells")


def test_sort_invariants(cuda_device, channel_cfg):
    ps, _ = _pair(channel_cfg)
    n = channel_cfg.n
    sp = ps.sortpart()
    assert np.array_equal(np.sort(sp), np.arange(n))
    cur = ps.d["CurPos"].cpu().numpy()
    assert np.array_equal(cur[sp], np.arange(n))
    keys = ps.d["CubePart"].cpu().numpy()
    assert np.all(np.diff(keys) >= 0)
    bec = ps.d["BeginEndCube"].cpu().numpy()
    for k in np.unique(keys):
        b, e = bec[k]
        assert np.all(keys[b:e] == k) and (b == 0 or keys[b - 1] != k) and (e == n or keys[e] != k)


def test_neighbor_sets_bit_exact(cuda_device, channel_cfg):
    import torch
    from gpucell_gb300 import _lib
    ps, o = _pair(channel_cfg)
    _sync_oracle(ps, o)
    n = channel_cfg.n
    cnt = torch.zeros(n, dtype=torch.int32, device="cuda")
    h = torch.zeros(n, dtype=torch.int64, device="cuda")
    _lib.call("gc_debug_neighbor_stats", n, ps.p("TotalCoor"), ps.p("SortPart"), ps.p("BeginEndCube"),
              C.c_void_p(cnt.data_ptr()), C.c_void_p(h.data_ptr()))
    inv = ps.fetch()["slot_of"]
    gc = cnt.cpu().numpy()[inv]
    gh = h.cpu().numpy().view(np.uint64)[inv]
    oc, oh = o.neighbor_stats()
    assert np.array_equal(gc, oc)
    assert np.array_equal(gh, oh)
    assert oc.mean() > 50


def test_density(cuda_device, channel_cfg):
    ps, o = _pair(channel_cfg)
    ps.density()
    g = ps.fetch()
    o.call("density")
    mob = slice(channel_cfg.n_b1 + channel_cfg.n_b2, None)
    np.testing.assert_allclose(g["rho"][mob], o.rho[mob], rtol=2e-6)
    # Bound2 keeps DenInit ("bound2 density is assumed constant")
    wb = slice(channel_cfg.n_b1, channel_cfg.n_b1 + channel_cfg.n_b2)
    np.testing.assert_allclose(g["rho"][wb], o.rho[wb], rtol=0)


def test_eos(cuda_device, channel_cfg):
    ps, o = _pair(channel_cfg)
    ps.eos()
    g = ps.fetch()
    o.call("eos")
    c2 = channel_cfg.phys.sound1 ** 2
    np.testing.assert_allclose(g["press"], o.press, atol=2e-6 * c2 * channel_cfg.den_init)


def test_integrator_stages(cuda_device, channel_cfg):
    ps, o = _pair(channel_cfg)
    ps.predict()
    g = ps.fetch()
    o.call("predict")
    np.testing.assert_allclose(g["vel"], o.vel, atol=1e-5)
    np.testing.assert_allclose(g["velhalf"], o.velhalf, atol=1e-5)
    ps.correct()
    g = ps.fetch()
    o.call("correct")
    np.testing.assert_allclose(g["vel"], o.vel, atol=1e-5)
    ps.update_coor()
    g = ps.fetch()
    o.call("update_coor")
    np.testing.assert_allclose(g["pos"], o.pos, atol=1e-5)
    # push some particles across the periodic faces
    st = _sync_oracle(ps, o)
    pos = st["pos"].astype(np.float64)
    L = float(channel_cfg.bbox[1] - channel_cfg.bbox[0])
    mob = np.arange(channel_cfg.n) >= channel_cfg.n_b1 + channel_cfg.n_b2
    pos[mob, 0] += 0.3 * L
    ps.set_state(pos=pos)
    o.set(pos=pos.astype(np.float32).astype(np.float64))
    ps.periodic()
    g = ps.fetch()
    o.call("periodic")
    np.testing.assert_allclose(g["pos"], o.pos, atol=1e-5)
    assert np.array_equal(g["nthro"], o.nthro) and np.abs(g["nthro"]).sum() > 0


def test_bound2_velocity(cuda_device, channel_cfg):
    ps, o = _pair(channel_cfg, wall_vel=0.5)
    ps.predict()                       # the wall velocity reads the caller's VelHalf pointer
    _sync_oracle(ps, o)
    ps.bound2_vel()
    g = ps.fetch()
    o.call("bound2_vel")
    wb = slice(channel_cfg.n_b1, channel_cfg.n_b1 + channel_cfg.n_b2)
    np.testing.assert_allclose(g["vel"][wb], o.vel[wb], atol=1e-5)


@pytest.mark.parametrize("noise", [False, True])
def test_sdpd_force(cuda_device, channel_cfg, noise):
    from gpucell_gb300 import _lib
    ps, o = _pair(channel_cfg, noise=noise)
    _lib.call("gc_set_step", 17)
    o.st.step = 17
    ps.sdpd_force()
    g = ps.fetch()
    o.call("sdpd_force")
    _force_close(g["force"], o.force, o.force_scale(o.SCALE_SDPD), what="SDPD force")


def test_repulsion_and_body_force(cuda_device, channel_cfg):
    ps, o = _pair(channel_cfg)
    # move some fluid close to the Bound1 layer so the repulsion acts
    st = _state(channel_cfg)
    ymin = float(channel_cfg.bbox[2])
    fl = np.arange(channel_cfg.n_b1 + channel_cfg.n_b2, channel_cfg.n_cell_start)
    pos = st["pos"].copy()
    pick = fl[:200]
    pos[pick, 1] = ymin - 1.0 + 0.15
    pos = pos.astype(np.float32).astype(np.float64)
    st["pos"] = pos
    ps.set_state(**st)
    ps.con_cube_list()
    o.set(**st)
    ps.rep_force()
    g = ps.fetch()
    o.call("rep_force")
    f0 = np.linalg.norm(st["force"], axis=1)     # the repulsion adds to the forces already there
    _force_close(g["force"], o.force, f0 + o.force_scale(o.SCALE_REP), what="repulsion")
    assert np.abs(g["force"] - st["force"]).max() > 0
    ps.ext_force(1)
    g = ps.fetch()
    o.call("ext_force")
    _force_close(g["force"], o.force, f0 + o.force_scale(o.SCALE_REP | o.SCALE_BODY), what="repulsion + body force")


def test_membrane_setup(cuda_device, channel_cfg):
    ps, o = _pair(channel_cfg)
    g = ps.fetch()
    np.testing.assert_allclose(g["RefEdgeLen"], o.refedgelen, rtol=1e-6)
    np.testing.assert_allclose(g["MaxRefEdgeLen"], o.maxrefedgelen, rtol=1e-6)
    np.testing.assert_allclose(g["PerLenWLC"], o.perlen, rtol=1e-5)
    np.testing.assert_allclose(g["HPow"], o.hpow, rtol=1e-5)
    np.testing.assert_allclose(g["HBending"], o.hbending, rtol=1e-6)
    np.testing.assert_allclose(np.cos(g["RefTriAngle"]), np.cos(o.refangle), atol=1e-5)
    np.testing.assert_allclose(np.sin(g["RefTriAngle"]), np.sin(o.refangle), atol=1e-5)
    np.testing.assert_allclose(g["RefArea_Para"][0], o.refarea[0], rtol=2e-6)
    np.testing.assert_allclose(g["RefVol_Para"][0], o.refvol[0], rtol=2e-6)


def test_geometry_and_deformation_force(cuda_device, channel_cfg):
    ps, o = _pair(channel_cfg, seed=3)
    ps.cal_geo_para()
    ps.d["TotalForce"].zero_()
    ps.def_force()
    g = ps.fetch()
    o.force[:] = 0
    o.call("geo", 0)
    o.call("def_force")
    np.testing.assert_allclose(g["Area"], o.area, rtol=2e-6)
    np.testing.assert_allclose(g["Vol"], o.vol, rtol=2e-6)
    np.testing.assert_allclose(g["TriArea"], o.triarea, rtol=1e-5)
    np.testing.assert_allclose(g["TriNorDir"], o.trinormal, atol=1e-5)
    np.testing.assert_allclose(g["TriCenter"], o.tricenter, atol=1e-5)
    np.testing.assert_allclose(g["ParArea"], o.pararea, rtol=1e-5)
    sc = o.force_scale(o.SCALE_MEMB)
    cs = channel_cfg.n_cell_start
    _force_close(g["DefForce"], o.defforce, sc[cs:], what="deformation force")
    _force_close(g["force"], o.force, sc, what="force")


def test_aggregation_force(cuda_device, two_cell_cfg):
    ps, o = _pair(two_cell_cfg, seed=4)
    ps.cal_geo_para()
    ps.d["TotalForce"].zero_()
    ps.agg_force()
    g = ps.fetch()
    o.force[:] = 0
    o.call("geo", 0)
    o.call("agg_force")
    assert np.abs(o.aggforce).max() > 0
    sc = o.force_scale(o.SCALE_MORSE)
    cs = two_cell_cfg.n_cell_start
    _force_close(g["AggForce"], o.aggforce, sc[cs:], what="aggregation force")
    _force_close(g["force"], o.force, sc, what="force")


def test_full_steps_track_the_oracle(cuda_device, channel_cfg):
    """Three complete steps in the reference order (noise off), starting from
    rest: positions within 1e-5, velocities within 1e-4 of their scale."""
    from gpucell_gb300.host import ParticleSystem
    from oracle.binding import Oracle
    cfg = channel_cfg
    ps = ParticleSystem(cfg, noise=False)
    o = Oracle(cfg, noise=False)
    o.setup()
    for _ in range(3):
        ps.update()
        o.step()
    g = ps.fetch()
    np.testing.assert_allclose(g["pos"], o.pos, atol=1e-5)
    vs = np.abs(o.vel).max()
    assert np.abs(g["vel"] - o.vel).max() <= 1e-4 * vs
    np.testing.assert_allclose(g["Area"], o.area, rtol=1e-5)
    np.testing.assert_allclose(g["Vol"], o.vol, rtol=1e-5)
