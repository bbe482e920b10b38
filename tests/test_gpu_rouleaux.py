"""Rouleaux found on the GPU (gc_ensemble_rouleaux) against an all-pairs
search of the stored membrane positions in numpy with the same FP32
arithmetic (difference, minimum image, squared distance rounded per
operation): identical labels and sizes for several contact distances, on a
periodic suspension whose cells cross the box faces, on a two-cell rouleau
in Couette flow, and per system of an ensemble."""
import numpy as np
import pytest

from gpucell_gb300 import generator as gen

pytestmark = pytest.mark.gpu


def _numpy_rouleaux(cfg, pos, contact):
    from gpucell_gb300 import rouleaux
    lo = cfg.bbox[0::2].astype(np.float32)
    hi = cfg.bbox[1::2].astype(np.float32)
    L = (hi - lo).astype(np.float32)
    half = (np.float32(0.5) * L).astype(np.float32)
    c2 = np.float32(contact) * np.float32(contact)
    m = pos[cfg.n_cell_start:].astype(np.float32)
    ends = np.cumsum(cfg.npar)
    starts = ends - cfg.npar
    pairs = []
    for a in range(cfg.ncell):
        xa = m[starts[a]:ends[a]]
        for b in range(a + 1, cfg.ncell):
            xb = m[starts[b]:ends[b]]
            d = (xa[:, None, :] - xb[None, :, :]).astype(np.float32)
            for k in range(3):
                if cfg.pmask & (1 << k):
                    dk = d[..., k]
                    dk = np.where(dk > half[k], dk - L[k], np.where(dk < -half[k], dk + L[k], dk))
                    d[..., k] = dk.astype(np.float32)
            r2 = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]).astype(np.float32) + d[..., 2] * d[..., 2]
            if (r2.astype(np.float32) < c2).any():
                pairs.append((a, b))
    return rouleaux.from_pairs(cfg.ncell, pairs)


def _check(fs, cfg, pos, contacts, sys=0):
    sizes_seen = []
    for c in contacts:
        label, size = fs.rouleaux(c, sys)
        want_label, want_size = _numpy_rouleaux(cfg, pos, c)
        assert np.array_equal(label, want_label), c
        assert np.array_equal(size, want_size), c
        sizes_seen.append(sorted(size.tolist(), reverse=True))
    return sizes_seen


def test_suspension_rouleaux_match_all_pairs(cuda_device):
    from gpucell_gb300.fused import FusedSystem
    cfg = gen.suspension(nx=36, ny=36, nz=36, ncells=10, subdiv=3, hematocrit=0.2, seed=21)
    fs = FusedSystem(cfg, noise=True)
    fs.step(20, 1)
    pos = fs.fetch()["pos"]
    # the stored positions are wrapped into the box: a cell that crosses a
    # face spans more than its extent taken as minimum images
    m = pos[cfg.n_cell_start:].astype(np.float64)
    L = (cfg.bbox[1::2] - cfg.bbox[0::2]).astype(np.float64)
    crossing = 0
    for e, n in zip(np.cumsum(cfg.npar), cfg.npar):
        x = m[e - n:e]
        d = x - x[0]
        d -= L * np.rint(d / L)
        crossing += int((np.ptp(x, axis=0) > np.ptp(d, axis=0) + 1e-3).any())
    assert crossing > 0, "no cell crosses a box face"
    seen = _check(fs, cfg, pos, [0.05, 0.3, 0.8, 1.5, 3.0])
    print("\nrouleau sizes by contact distance:", seen)
    assert len(set(map(tuple, seen))) > 1   # the distances give different pictures


def test_couette_rouleau_of_two(cuda_device):
    from gpucell_gb300.fused import FusedSystem
    cfg = gen.couette(nx=36, ny=18, nz=24, ncells=2, subdiv=2, cell_diameter=3.0, shear_rate=0.5, seed=31)
    fs = FusedSystem(cfg, noise=False)
    fs.step(10, 1)
    pos = fs.fetch()["pos"]
    seen = _check(fs, cfg, pos, [0.1, 0.5, 1.0, 2.5])
    assert seen[-1] == [2]


def test_ensemble_rouleaux_per_system(cuda_device):
    from gpucell_gb300.fused import Ensemble
    cfgs = [gen.suspension(nx=30, ny=30, nz=30, ncells=k, subdiv=2, hematocrit=0.25, seed=40 + k)
            for k in (0, 6, 3)]
    ens = Ensemble(cfgs, noise=True)
    ens.step(10, 1)
    for s, cfg in enumerate(cfgs):
        pos = ens.fetch(s)["pos"]
        if cfg.ncell == 0:
            label, size = ens.rouleaux(1.0, s)
            assert label.size == 0 and size.size == 0
            continue
        _check(ens, cfg, pos, [0.2, 1.0], sys=s)
