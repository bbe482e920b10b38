"""The host-side checks bench.py applies to GPU results, against the FP64
oracle: cell_geometry_fp64 (area and volume of every cell from stored FP32
positions and crossing counts) equals the oracle's geometry pass on the same
wrapped state, for cells that cross the periodic faces."""
import os
import sys

import numpy as np

from gpucell_gb300 import generator as gen

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def test_cell_geometry_matches_the_oracle():
    import bench
    from oracle.binding import Oracle
    cfg = gen.constriction(nx=60, ny=30, nz=24, ncells=4, subdiv=2, cell_diameter=2.4, layout="random", seed=9)
    lo = cfg.bbox[0::2].astype(np.float64)
    L = cfg.bbox[1::2].astype(np.float64) - lo
    per = np.array([(cfg.pmask >> k) & 1 for k in range(3)], bool)
    x = cfg.coor.astype(np.float64)
    x[cfg.n_cell_start:, 0] += 0.55 * L[0]   # move the cells so that some cross the x and z faces
    x[cfg.n_cell_start:, 2] += 0.45 * L[2]
    nthro = np.where(per, np.floor((x - lo) / L), 0).astype(np.int32)
    wrapped = (x - nthro * L).astype(np.float32)
    assert (nthro[cfg.n_cell_start:] != 0).any(), "no vertex outside the box"
    area, vol = bench.cell_geometry_fp64(cfg, wrapped, nthro)
    o = Oracle(cfg, noise=False)
    o.set(pos=wrapped.astype(np.float64), nthro=nthro)
    o.call("geo", 0)
    np.testing.assert_allclose(area, o.area, rtol=1e-12)
    np.testing.assert_allclose(vol, o.vol, rtol=1e-12)
