"""Reproducibility, checkpoint and restart of the fused step.

* Two runs of the same configuration (cells, noise on, list rebuilds) give
  bit-identical state: every sum on the path has a fixed order (membrane
  forces are gathered per vertex, not accumulated with float atomics).
* A run restored from a checkpoint continues bit for bit as the original run
  does, through list rebuilds, with the restored handle created at another
  skin (the checkpoint's skin is adopted); right after the restore the
  stored state equals the state at the checkpoint.
* A checkpoint of another configuration, a file that is not one, or one of
  the wrong length is refused with an error, and a refused handle steps on
  exactly as if the restore had not been asked for.
"""
import numpy as np
import pytest

from gpucell_gb300 import generator as gen

pytestmark = pytest.mark.gpu

KEYS = ("pos", "vel", "rho", "press", "force", "velhalf", "nthro", "Area64", "Vol64", "DefForce", "AggForce",
        "TriNorDir", "ParArea")


def _cfg():
    phys = gen.Physics(ext_force=0.02, sur_energy=2e-3, sca_fac=1.5, zero_len=0.3, max_cut=1.2)
    return gen.suspension(nx=30, ny=18, nz=18, ncells=2, subdiv=2, hematocrit=0.12, seed=4, phys=phys)


def _same(a, b, keys=KEYS):
    for k in keys:
        assert np.array_equal(a[k], b[k]), k


def test_two_runs_are_bit_identical(cuda_device):
    from gpucell_gb300.fused import FusedSystem
    cfg = _cfg()
    out = []
    for _ in range(2):
        fs = FusedSystem(cfg, noise=True, skin=0.03)
        fs.step(40, 1)
        assert fs.stats()["rebuilds"] >= 2
        out.append(fs.fetch())
        fs.close()
    _same(out[0], out[1])


def test_restart_continues_bit_for_bit(cuda_device, tmp_path):
    from gpucell_gb300.fused import FusedSystem
    cfg = _cfg()
    path = tmp_path / "state.ckpt"
    a = FusedSystem(cfg, noise=True, skin=0.03)
    a.step(25, 1)
    at_ckpt = a.fetch()
    a.checkpoint(path)
    r0 = a.stats()["rebuilds"]
    a.step(30, 1)
    assert a.stats()["rebuilds"] > r0          # the continuation crosses list rebuilds
    want = a.fetch()
    b = FusedSystem(cfg, noise=True, skin=0.1)
    b.restore(path)
    assert b.options()["skin"] == pytest.approx(0.03)
    _same(b.fetch(), at_ckpt, ("pos", "vel", "rho", "press", "force", "velhalf", "nthro", "Area64", "Vol64"))
    b.step(30, 1)
    _same(b.fetch(), want)
    assert b.flags() == 0


def test_restore_refuses_other_files(cuda_device, tmp_path):
    from gpucell_gb300 import _lib
    from gpucell_gb300.fused import FusedSystem
    a = FusedSystem(_cfg(), noise=True)
    a.checkpoint(tmp_path / "a.ckpt")
    other = FusedSystem(gen.suspension(nx=16, ny=16, nz=16, ncells=0, seed=5), noise=True)
    with pytest.raises(_lib.GcError, match="another configuration"):
        other.restore(tmp_path / "a.ckpt")
    (tmp_path / "junk").write_bytes(b"not a checkpoint" * 16)
    with pytest.raises(_lib.GcError, match="not a checkpoint"):
        a.restore(tmp_path / "junk")
    with pytest.raises(_lib.GcError, match="cannot open"):
        a.restore(tmp_path / "missing.ckpt")


def test_ensemble_with_aggregation_restarts_bit_for_bit(cuda_device, tmp_path):
    """An ensemble (a Couette rouleau and a suspension, Morse aggregation on
    in both) checkpointed and continued across list rebuilds in a new handle
    matches the uninterrupted run bit for bit, aggregation forces included."""
    from gpucell_gb300.fused import Ensemble
    cou = gen.couette(nx=36, ny=18, nz=24, ncells=2, subdiv=2, cell_diameter=3.0, shear_rate=0.5, seed=31)
    sus = gen.suspension(nx=30, ny=24, nz=24, ncells=2, subdiv=2, hematocrit=0.08, seed=4, phys=cou.phys)
    cfgs = [cou, sus]
    path = tmp_path / "ens.ckpt"
    a = Ensemble(cfgs, noise=True, skin=0.05)
    a.step(20, 0)
    a.checkpoint(path)
    r0 = a.stats()["rebuilds"]
    a.step(25, 0)
    assert a.stats()["rebuilds"] > r0
    want = [a.fetch(s) for s in range(2)]
    b = Ensemble(cfgs, noise=True)
    b.restore(path)
    b.step(25, 0)
    for s in range(2):
        got = b.fetch(s)
        _same(got, want[s], ("pos", "vel", "force", "rho", "nthro", "Area64", "Vol64", "AggForce"))
    assert np.abs(want[0]["AggForce"]).max() > 0
    assert b.flags() == 0
    a.close()
    b.close()


def test_refused_restore_leaves_the_handle_as_it_was(cuda_device, tmp_path):
    from gpucell_gb300 import _lib
    from gpucell_gb300.fused import FusedSystem
    cfg = _cfg()
    a = FusedSystem(cfg, noise=True, skin=0.03)
    a.step(10, 1)
    a.checkpoint(tmp_path / "a.ckpt")
    data = (tmp_path / "a.ckpt").read_bytes()
    (tmp_path / "short.ckpt").write_bytes(data[:-4])
    (tmp_path / "long.ckpt").write_bytes(data + bytes(8))
    b = FusedSystem(cfg, noise=True, skin=0.1)   # another skin: a refused file's is not adopted
    twin = FusedSystem(cfg, noise=True, skin=0.1)
    for bad in ("short.ckpt", "long.ckpt"):
        with pytest.raises(_lib.GcError, match="bytes, a checkpoint of this configuration"):
            b.restore(tmp_path / bad)
    assert b.options()["skin"] == pytest.approx(0.1)
    b.step(30, 1)
    twin.step(30, 1)
    assert b.stats()["rebuilds"] == twin.stats()["rebuilds"]
    _same(b.fetch(), twin.fetch())
    assert b.flags() == 0
