"""Ensembles, captured steps and the autotuner of the fused step.

* An ensemble of unlike systems (a walled channel with a cell, a periodic
  suspension, a plain fluid box) stepped by the same launches follows each
  system run alone: the pair noise is keyed by the system's own ids and
  seed, so the only differences are FP32 summation order after rebuilds
  that the other systems triggered.  Positions within 1e-5, velocities and
  forces within 1e-4 of their largest magnitude, membrane area/volume within
  1e-6 relative (FP64 sums).
* Captured steps (each step one CUDA graph, rebuild decided on the device)
  follow the host-driven steps to the same tolerances, for one system and
  for an ensemble, and count the same rebuilds when started alike.
* The autotuner returns one of its candidates, leaves the state as it found
  it (positions and velocities bit-identical), and the run that follows
  matches an untuned run within the same tolerances.
"""
import numpy as np
import pytest

from gpucell_gb300 import generator as gen

pytestmark = pytest.mark.gpu


def _close_rel(got, want, tol):
    scale = max(float(np.abs(want).max()), 1e-30)
    assert float(np.abs(got - want).max()) <= tol * scale


def _systems():
    a = gen.small_channel(seed=3)
    b = gen.suspension(nx=30, ny=18, nz=18, ncells=2, subdiv=2, hematocrit=0.12, seed=4,
                       phys=gen.Physics(ext_force=0.01, seed=77))
    c = gen.suspension(nx=16, ny=16, nz=16, ncells=0, seed=5, phys=gen.Physics(ext_force=0.03, seed=91))
    return [a, b, c]


def _compare(got, want, cells=True):
    np.testing.assert_allclose(got["pos"], want["pos"], atol=1e-5)
    _close_rel(got["vel"], want["vel"], 1e-4)
    _close_rel(got["force"], want["force"], 1e-4)
    _close_rel(got["rho"], want["rho"], 1e-5)
    assert np.array_equal(got["nthro"], want["nthro"])
    if cells and "Area64" in want:
        np.testing.assert_allclose(got["Area64"], want["Area64"], rtol=1e-6)
        np.testing.assert_allclose(got["Vol64"], want["Vol64"], rtol=1e-6)
        np.testing.assert_allclose(got["TriNorDir"], want["TriNorDir"], atol=1e-4)


@pytest.mark.parametrize("graph", [False, True])
def test_ensemble_follows_single_runs(cuda_device, graph):
    from gpucell_gb300.fused import Ensemble, FusedSystem
    cfgs = _systems()
    ens = Ensemble(cfgs, noise=True, graph=graph)
    ens.step(12, 1)
    for s, cfg in enumerate(cfgs):
        solo = FusedSystem(cfg, noise=True)
        solo.step(12, 1)
        _compare(ens.fetch(s), solo.fetch())
        solo.close()
    assert ens.flags() == 0
    ens.close()


def test_ensemble_whole_store_concatenates_systems(cuda_device):
    import ctypes as C
    from gpucell_gb300 import _lib
    from gpucell_gb300.fused import Ensemble, _ptr
    cfgs = _systems()
    ens = Ensemble(cfgs, noise=False)
    ens.step(3, 1)
    n = sum(c.n for c in cfgs)
    pos = np.empty((n, 3), np.float32)
    _lib.call("gc_fused_store", ens.h, _ptr(pos), *([C.c_void_p(0)] * 6), 0)
    off = 0
    for s, c in enumerate(cfgs):
        assert np.array_equal(pos[off:off + c.n], ens.fetch(s)["pos"])
        off += c.n
    ns, npart = C.c_int(), C.c_longlong()
    _lib.call("gc_ensemble_size", ens.h, C.byref(ns), C.byref(npart))
    assert (ns.value, npart.value) == (3, n)


def test_ensemble_rejects_unlike_physics(cuda_device):
    from gpucell_gb300 import _lib
    from gpucell_gb300.fused import Ensemble
    a = gen.suspension(nx=16, ny=16, nz=16, ncells=0, seed=5)
    b = gen.suspension(nx=16, ny=16, nz=16, ncells=0, seed=6, phys=gen.Physics(shear_vis=20.0))
    with pytest.raises(_lib.GcError, match="other physics"):
        Ensemble([a, b])


@pytest.mark.parametrize("ensemble", [False, True])
def test_captured_steps_follow_host_steps(cuda_device, ensemble):
    from gpucell_gb300.fused import Ensemble, FusedSystem
    if ensemble:
        cfgs = _systems()
        host, capt = Ensemble(cfgs, graph=False), Ensemble(cfgs, graph=True)
    else:
        cfgs = [gen.small_channel(seed=9)]
        host, capt = FusedSystem(cfgs[0], graph=False), FusedSystem(cfgs[0], graph=True)
    # one forced rebuild on both sides so that they start from the same lists
    host.set_options(skin=0.12)
    capt.set_options(skin=0.12)
    for _ in range(4):
        host.step(10, 1)
        capt.step(10, 1)
    for s in range(len(cfgs)):
        got = capt.fetch(s) if ensemble else capt.fetch()
        want = host.fetch(s) if ensemble else host.fetch()
        _compare(got, want)
    sh, sc = host.stats(), capt.stats()
    assert sc["steps"] == sh["steps"] == 40
    assert sc["rebuilds"] >= 1
    assert capt.options()["graph"] and not host.options()["graph"]
    assert capt.flags() == 0


@pytest.mark.parametrize("room", ["default", "exact"])
def test_captured_steps_with_aggregation_follow_host_steps(cuda_device, monkeypatch, room):
    """The Morse aggregation inside captured steps (its lists rebuilt in the
    captured rebuilds, the listed pairs each step): a two-cell rouleau in
    Couette flow follows the host-driven steps, aggregation forces included.
    With the Morse lists allocated to fit exactly ("exact",
    GPUCELL_MORSE_ROOM=1), a captured rebuild whose lists grow overflows
    them; the host runs those steps again with room, and the results are
    the same."""
    from gpucell_gb300.fused import FusedSystem
    if room == "exact":
        monkeypatch.setenv("GPUCELL_MORSE_ROOM", "1")
    cfg = gen.couette(nx=36, ny=18, nz=24, ncells=2, subdiv=2, cell_diameter=3.0, shear_rate=0.5, seed=31)
    host, capt = FusedSystem(cfg, graph=False), FusedSystem(cfg, graph=True)
    skin = 0.12 if room == "default" else 0.02
    host.set_options(skin=skin)
    capt.set_options(skin=skin)
    for _ in range(3):
        host.step(10, 1)
        capt.step(10, 1)
    got, want = capt.fetch(), host.fetch()
    _compare(got, want)
    assert np.abs(want["AggForce"]).max() > 0
    np.testing.assert_allclose(got["AggForce"], want["AggForce"], rtol=0, atol=1e-5 * np.abs(want["AggForce"]).max())
    assert capt.stats()["rebuilds"] >= 1 and capt.flags() == 0


def test_captured_steps_count_launches(cuda_device):
    from gpucell_gb300 import _lib
    from gpucell_gb300.fused import FusedSystem
    fs = FusedSystem(gen.small_channel(seed=9), graph=True)
    fs.step(2, 1)                      # capture
    l0 = _lib.launch_count()
    fs.step(10, 1)
    got = _lib.launch_count() - l0
    # at least the five per-step kernels (prologue, integrate, condition,
    # density, force) for every replayed step
    assert got >= 50


def test_autotune_keeps_state_and_trajectory(cuda_device):
    from gpucell_gb300.fused import FusedSystem
    cfg = gen.suspension(nx=30, ny=18, nz=18, ncells=2, subdiv=2, hematocrit=0.12, seed=4)
    tuned, plain = FusedSystem(cfg, noise=True), FusedSystem(cfg, noise=True)
    tuned.step(5, 1)
    plain.step(5, 1)
    before = tuned.fetch()
    choice = tuned.autotune(trial_steps=6)
    after = tuned.fetch()
    assert np.array_equal(after["pos"], before["pos"])
    assert np.array_equal(after["vel"], before["vel"])
    _close_rel(after["rho"], before["rho"], 1e-5)
    assert choice["skin"] in (0.05, 0.075, 0.1, 0.15)
    assert choice["block"] in (64, 128, 256)
    assert choice["ms_per_step"] > 0
    assert tuned.options()["skin"] == choice["skin"]
    assert tuned.stats()["steps"] == 5
    tuned.step(10, 1)
    plain.step(10, 1)
    _compare(tuned.fetch(), plain.fetch())
    # the cache answers the same size class without trials
    again = FusedSystem(cfg, noise=True)
    cached = again.autotune(trial_steps=6, use_cache=True)
    assert cached["ms_per_step"] == 0.0
    assert {k: cached[k] for k in ("skin", "block", "compact", "graph")} == \
        {k: choice[k] for k in ("skin", "block", "compact", "graph")}


def test_smallest_periodic_system_in_an_ensemble(cuda_device):
    """A system in a box of five half-width cells along each periodic axis
    (L = 3.0, 729 particles: the radius-2 stencil then covers every cell of
    the box exactly once) beside a larger one steps as it does alone."""
    from gpucell_gb300.fused import Ensemble, FusedSystem
    tiny = gen.suspension(nx=9, ny=9, nz=9, ncells=0, seed=8, phys=gen.Physics(ext_force=0.02, seed=5))
    big = gen.suspension(nx=30, ny=18, nz=18, ncells=2, subdiv=2, hematocrit=0.12, seed=4,
                         phys=gen.Physics(ext_force=0.01, seed=77))
    assert tiny.n == 729 and abs(float(tiny.bbox[1] - tiny.bbox[0]) - 3.0) < 1e-5
    ens = Ensemble([big, tiny], noise=True)
    alone = FusedSystem(tiny, noise=True)
    ens.step(20, 1)
    alone.step(20, 1)
    _compare(ens.fetch(1), alone.fetch(), cells=False)
    assert ens.flags() == 0 and alone.flags() == 0
    ens.close()
    alone.close()
