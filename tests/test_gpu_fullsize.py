"""The 4.2M-particle suspension of the benchmark (256 x 128 x 128 sites, 200
cells of 2562 vertices, noise on), where the FP64 oracle is too slow to
step, checked through properties that hold at any size:

* two runs of the same input are bit-identical (every sum has a fixed
  order), across list rebuilds;
* the total momentum stays at zero to rounding: the pair forces, random
  ones included, and the membrane forces are antisymmetric, and there is no
  body force (|P| below 1e-5 of the thermal momentum scale sqrt(2 E M));
* the GPU's FP64 per-cell areas and volumes equal an FP64 evaluation on the
  host from the stored positions and crossing counts (relative 1e-6), and
  stay within 2 % of their set-up values;
* every stored value is finite and no device flag is raised.
"""
import os
import sys

import numpy as np
import pytest

from gpucell_gb300 import generator as gen

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

STEPS = 40


@pytest.fixture(scope="module")
def cfg2():
    return gen.suspension(seed=12345)


def _run(cfg):
    from gpucell_gb300.fused import FusedSystem
    fs = FusedSystem(cfg, noise=True, skin=0.075)
    a0 = fs.fetch()
    fs.step(STEPS, 1)
    out = fs.fetch()
    out["diag"] = fs.diagnostics()
    out["stats"] = fs.stats()
    out["flags"] = fs.flags()
    out["Area0"], out["Vol0"] = a0["Area64"], a0["Vol64"]
    fs.close()
    return out


def test_full_size_properties(cuda_device, cfg2):
    import bench
    assert cfg2.n == 4194304 and cfg2.ncell == 200
    a = _run(cfg2)
    b = _run(cfg2)
    assert a["flags"] == 0 and b["flags"] == 0
    assert a["stats"]["rebuilds"] >= 2   # the runs cross list rebuilds
    for k in ("pos", "vel", "force", "rho", "nthro", "Area64", "Vol64"):
        assert np.array_equal(a[k], b[k]), k
    for k in ("pos", "vel", "force", "rho", "press"):
        assert np.isfinite(a[k]).all(), k
    d = a["diag"]
    scale = np.sqrt(2.0 * d["kinetic_energy"] * cfg2.phys.mass * d["moving"])
    print(f"\n|P| / sqrt(2 E M) = {np.linalg.norm(d['momentum']) / scale:.2e}, kT = {d['temperature']:.3f}")
    assert np.linalg.norm(d["momentum"]) < 1e-5 * scale
    ha, hv = bench.cell_geometry_fp64(cfg2, a["pos"], a["nthro"])
    ea, ev = np.abs(a["Area64"] / ha - 1).max(), np.abs(a["Vol64"] / hv - 1).max()
    print(f"cell area / volume vs FP64 host: {ea:.2e} / {ev:.2e}")
    assert ea < 1e-6 and ev < 1e-6
    assert np.abs(a["Area64"] / a["Area0"] - 1).max() < 0.02
    assert np.abs(a["Vol64"] / a["Vol0"] - 1).max() < 0.02


def test_host_load_and_store_in_pieces_round_trip(cuda_device, cfg2):
    """Host loads and stores of a million particles or more go in four
    pieces (copies of one piece beside the conversion kernel of the next):
    a state loaded in place comes back bit for bit, each array in the
    caller's order, including the pieces' edges."""
    from gpucell_gb300.fused import FusedSystem
    rng = np.random.default_rng(5)
    n = cfg2.n
    assert n >= 1 << 20   # the pieced path
    fs = FusedSystem(cfg2, noise=False)
    state = {"pos": cfg2.coor.astype(np.float32),
             "vel": rng.standard_normal((n, 3)).astype(np.float32),
             "velhalf": rng.standard_normal((n, 3)).astype(np.float32),
             "force": rng.standard_normal((n, 3)).astype(np.float32),
             "nthro": rng.integers(-3, 4, size=(n, 3)).astype(np.int32)}
    fs.load(state["pos"], state["vel"], state["velhalf"], state["force"], state["nthro"])
    got = fs.fetch()
    fs.close()
    for k, want in state.items():
        assert np.array_equal(got[k], want), k
