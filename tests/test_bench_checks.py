"""The host-side checks bench.py applies to GPU results: cell_geometry_fp64
(area and volume of every cell from stored FP32 positions and crossing
counts) equals the FP64 oracle's geometry pass on the same wrapped state, for
cells that cross the periodic faces; the clock record is read from
nvidia-smi's samples with their throttle reasons; the metric is named by the
size it ran at."""
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


class _FakeSampler:
    """Stands in for the nvidia-smi process the sampler started."""

    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def test_clock_samples_are_read_with_their_throttle_reasons(tmp_path):
    """The bench line's `clocks` record: SM clocks of the benchmarked GPU only,
    unreadable samples skipped, every throttle reason that was active in any
    sample reported (a run with hw_slowdown or a thermal slowdown is rejected
    by whoever reads the line; sw_power_cap is kept and noted)."""
    import bench
    lines = [
        "0, 2070, 2070, 900.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 1980, 2070, 1400.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "1, 1200, 2070, 300.0, 0x0000000000000008, Active, Not Active, Not Active, Not Active",
        "0, [N/A], 2070, 950.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 2070, 2070, 950.0, 0x0000000000000040, Not Active, Active, Not Active, Not Active",
    ]
    s = bench.ClockSampler()
    s.path = str(tmp_path / "clocks.csv")
    with open(s.path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    s.fh = open(os.devnull, "w")
    s.proc = _FakeSampler()
    rec = s.stop(gpu_index=0)
    assert rec == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "samples": 3,
                   "reasons": ["hw_thermal_slowdown", "sw_power_cap"], "source": "nvidia-smi", "interval_ms": 50}
    assert not os.path.exists(s.path)
    assert bench.ClockSampler().stop() is None   # never started: no record


class _FakeNvml:
    """Stands in for NVML: SM clocks 1980 then 2070 MHz, sw_power_cap then
    hw_slowdown + sw_power_cap active."""

    def __init__(self):
        self.n = 0
        self.shut = False

    def nvmlDeviceGetClockInfo(self, h, kind, p):
        assert kind == 1
        p._obj.value = 1980 if self.n == 0 else 2070
        return 0

    def nvmlDeviceGetMaxClockInfo(self, h, kind, p):
        p._obj.value = 2070
        return 0

    def nvmlDeviceGetCurrentClocksEventReasons(self, h, p):
        p._obj.value = 0x4 if self.n == 0 else 0xC
        self.n += 1
        return 0

    def nvmlShutdown(self):
        self.shut = True
        return 0


def test_nvml_clock_samples_are_taken_in_a_thread():
    """The NVML sampler: one sample at least before the timed region
    starts, the reason bits named, NVML shut down at the end."""
    import time

    import bench
    lib = _FakeNvml()
    s = bench.ClockSampler(interval_ms=5)
    s._start_nvml(lib, object())
    assert len(s.samples) >= 1
    time.sleep(0.05)
    rec = s.stop()
    assert lib.shut and rec["source"] == "nvml" and rec["interval_ms"] == 5
    assert rec["samples"] >= 2 and rec["sm_max_mhz"] == 2070.0
    assert rec["reasons"] == ["hw_slowdown", "sw_power_cap"]


def test_metric_name_follows_the_workload_size():
    import bench
    assert bench.metric_name(4194304) == bench.METRIC
    assert bench.metric_name(524288) == "particle-steps/s on 524288-particle RBC suspension"


def test_roofline_follows_the_algorithmic_byte_formula():
    """roofline.frac of the bench line is particle-steps/s x B_alg / N / the
    HBM peak, with B_alg = 352 N + 16 N_tri + 32 N_edge + 28 N_vert (1.556 GB
    per step on the 4.2M-particle suspension)."""
    import types
    import bench
    cfg = types.SimpleNamespace(n=4194304, ntri=1024000, nedge=1536000, ncp=512400)
    b_alg = bench.plain_bytes_per_step(cfg)
    assert abs(b_alg / 1e9 - 1.556) < 1e-3
    ms = 4.78
    roof, kern, issue, fp32 = bench.rooflines(cfg, ms, 2.87, 1.1, 143.0, 6789.3, "measured", None, True)
    value = cfg.n / (ms / 1e3)
    assert abs(roof["frac"] - value * b_alg / cfg.n / 1e9 / 6789.3) < 1e-12
    assert roof["bound"] == "hbm" and roof["unit"] == "GB/s" and roof["peak"] == 6789.3
    assert abs(kern["fk_force"]["alg_bytes_per_launch"] - 72 * cfg.n) < 1
    assert kern["fk_force"]["streamed_bytes_per_launch"] > kern["fk_force"]["alg_bytes_per_launch"]
    assert 0 < issue["frac"] < 2 and 0 < fp32["frac"] < 2
