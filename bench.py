#!/usr/bin/env python
"""Throughput of the SDPD + membrane timestep on the 4.2M-particle red-cell
suspension (256x128x128 particles, 200 cells of 2562 vertices, hematocrit
20 %, periodic, thermal noise on).

Prints one JSON line.  `value` is particle-steps/s of the fused step with the
state resident in HBM; `plain_fp32` is the reference-structured FP32 step
(one kernel per boundary entry point) on the same workload; `e2e` is the
fused step with the state copied host->device before and device->host after
every step (pinned buffers); `roofline` describes the dominant kernel, timed
live with CUDA events; `cpu_baseline` is the FP64 CPU restatement of the
method timed on this machine's cores on a bounded sample.

    python bench.py [--steps K] [--warmup W] [--skin S] [--block B] [--no-plain]
    python bench.py --impl reference      # the CPU restatement alone
    torchrun --nproc-per-node N bench.py --gpus N   # independent replicas
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "particle-steps/s on 4.2M-particle RBC suspension"


def metric_name(n: int) -> str:
    """The headline metric's name for the full suspension; the size it ran at otherwise."""
    return METRIC if n == 4194304 else "particle-steps/s on %d-particle RBC suspension" % n
PEAKS_FALLBACK = {"hbm_gbs": 6800.0}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--skin", type=float, default=0.125,
                    help="Verlet skin in units of the cut-off (0.125: fastest of 0.075-0.175 over 100 and 300 steps)")
    ap.add_argument("--block", type=int, default=128)
    ap.add_argument("--tiles", action="store_true",
                    help="pair tiles (each pair once, both sides from one evaluation) instead of per-particle lists")
    ap.add_argument("--no-compact", dest="compact", action="store_false",
                    help="force pass iterates the skin lists instead of the per-step compact lists")
    ap.add_argument("--no-plain", dest="plain", action="store_false", help="skip the FP32 boundary-path timing")
    ap.add_argument("--no-engine", dest="engine", action="store_false",
                    help="skip the boundary entry points with the fused engine behind them")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-steps", type=int, default=10,
                    help="timed FP64 oracle steps of the CPU baseline (after one warm-up step)")
    ap.add_argument("--ref-steps-cap", type=int, default=30,
                    help="the reference arm times min(--steps, this) oracle steps")
    ap.add_argument("--ens-seq-steps", type=int, default=10,
                    help="steps per system of the sequential baselines of the ensemble")
    ap.add_argument("--no-variants", dest="variants", action="store_false",
                    help="skip timing the precision variants (plain FP32 positions, FP16 neighbour velocities) "
                         "and the pair tiles on the same workload")
    ap.add_argument("--no-configs", dest="configs", action="store_false",
                    help="skip the short cfg3 (sheared suspension) and cfg4 (constriction) legs")
    ap.add_argument("--config-steps", type=int, default=200, help="steps of the cfg3 and cfg4 legs")
    ap.add_argument("--small", action="store_true", help="a 1/8-size suspension (for quick checks)")
    ap.add_argument("--no-noise", dest="noise", action="store_false",
                    help="thermal noise off (for cost breakdowns; the reported workload has it on)")
    ap.add_argument("--graph", action="store_true", help="captured steps (one CUDA graph per step)")
    ap.add_argument("--tune", action="store_true", help="let the autotuner pick skin, block, compaction, graph")
    ap.add_argument("--tune-steps", type=int, default=20)
    ap.add_argument("--profile-steps", type=int, default=10, help="steps of the per-kernel timing pass")
    ap.add_argument("--no-ensemble", dest="ensemble", action="store_false",
                    help="skip the 64-suspension ensemble workload")
    ap.add_argument("--ensemble-only", action="store_true", help="only the ensemble workload")
    ap.add_argument("--ens-systems", type=int, default=64)
    ap.add_argument("--ens-steps", type=int, default=20)
    ap.add_argument("--no-parity", dest="parity", action="store_false",
                    help="skip the parity checks against the FP64 oracle (the workload itself, and a small channel)")
    ap.add_argument("--no-output", dest="output", action="store_false",
                    help="skip timing one output step (GPUCell's output files)")
    ap.add_argument("--rouleaux-run", action="store_true",
                    help="instead of the suspension: rouleau sizes of 64 cells in Couette flow (1.0M fluid "
                         "particles) tracked over --rouleaux-steps steps at three shear rates")
    ap.add_argument("--rouleaux-steps", type=int, default=20000)
    ap.add_argument("--rouleaux-every", type=int, default=1000)
    ap.add_argument("--rouleaux-contact", type=float, default=0.6)
    ap.add_argument("--shear-rates", type=str, default="0.005,0.05,0.5")
    ap.add_argument("--rouleaux-temp", type=float, default=0.1,
                    help="k_B T of the rouleaux run (the Morse adhesion of a cell contact is ~1.5 energy units)")
    ap.add_argument("--constriction-run", action="store_true",
                    help="instead of the suspension: 100 cells through a 2:1 constriction (2.0M particles), with "
                         "an FP64 host check of every cell's area and volume every --check-every steps")
    ap.add_argument("--constriction-steps", type=int, default=1000)
    ap.add_argument("--check-every", type=int, default=100)
    return ap.parse_args()


def workload(args, rank=0):
    from gpucell_gb300 import generator
    if args.small:
        return generator.suspension(nx=128, ny=64, nz=64, ncells=25, seed=12345 + rank), \
            dict(workload="rbc_suspension_small", nx=128, ny=64, nz=64, cells=25, vertices_per_cell=2562)
    return generator.suspension(seed=12345 + rank), \
        dict(workload="rbc_suspension", nx=256, ny=128, nz=128, cells=200, vertices_per_cell=2562)


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return PEAKS_FALLBACK, "fallback"


# Clock-event reason bits of NVML's public API (nvmlClocksEventReason*), the
# ones a bench line reports.
NVML_REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
                0x80: "hw_power_brake_slowdown"}


def _nvml():
    """NVML through ctypes (read-only queries), or None where the driver's
    library is absent."""
    import ctypes
    try:
        lib = ctypes.CDLL("libnvidia-ml.so.1")
    except OSError:
        return None
    if lib.nvmlInit_v2() != 0:
        return None
    return lib


def _nvml_handle(lib, device):
    """The NVML handle of CUDA device `device` (by PCI address when torch
    gives it, else by index)."""
    import ctypes
    h = ctypes.c_void_p()
    try:
        import torch
        p = torch.cuda.get_device_properties(device)
        bus = f"{p.pci_domain_id:08x}:{p.pci_bus_id:02x}:{p.pci_device_id:02x}.0".encode()
        if lib.nvmlDeviceGetHandleByPciBusId_v2(ctypes.c_char_p(bus), ctypes.byref(h)) == 0:
            return h
    except (AttributeError, RuntimeError, AssertionError):
        pass
    if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(device), ctypes.byref(h)) == 0:
        return h
    return None


def clock_record(samples, source, interval_ms):
    """The bench line's `clocks` record from (sm_mhz, sm_max_mhz, reasons)
    samples: median SM clock, the largest maximum clock, every throttle
    reason active in any sample."""
    if not samples:
        return None
    reasons = set()
    for _, _, r in samples:
        reasons |= set(r)
    return {"sm_mhz": statistics.median(x[0] for x in samples), "sm_max_mhz": max(x[1] for x in samples),
            "samples": len(samples), "reasons": sorted(reasons), "source": source, "interval_ms": interval_ms}


class ClockSampler:
    """SM clocks and throttle reasons of the benchmarked GPU during a timed
    region: NVML queried every `interval_ms` from a thread (the foreign calls
    release the GIL), or, where NVML cannot be loaded, nvidia-smi every 50 ms.
    Reading these settings changes nothing on the GPU."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, interval_ms=10):
        self.proc = None
        self.path = None
        self.thread = None
        self.interval_ms = interval_ms

    def start(self, device=None):
        if device is None:
            try:
                import torch
                device = torch.cuda.current_device()
            except (ImportError, RuntimeError, AssertionError):
                device = 0
        lib = _nvml()
        h = _nvml_handle(lib, device) if lib is not None else None
        if h is not None:
            self._start_nvml(lib, h)
        else:
            self._start_smi()

    def _start_nvml(self, lib, h):
        import ctypes  # noqa: F401 (the by-reference arguments below)
        import threading
        self.samples, self.stop_evt = [], threading.Event()
        have_events = hasattr(lib, "nvmlDeviceGetCurrentClocksEventReasons")
        reasons_fn = (lib.nvmlDeviceGetCurrentClocksEventReasons if have_events
                      else lib.nvmlDeviceGetCurrentClocksThrottleReasons)
        first = threading.Event()

        def run():
            sm, mx, r = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
            while not self.stop_evt.is_set():
                if (lib.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(sm)) == 0          # NVML_CLOCK_SM
                        and lib.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0
                        and reasons_fn(h, ctypes.byref(r)) == 0):
                    self.samples.append((float(sm.value), float(mx.value),
                                         [nm for bit, nm in NVML_REASONS.items() if r.value & bit]))
                first.set()
                self.stop_evt.wait(self.interval_ms / 1e3)
            first.set()

        self.lib = lib
        self.thread = threading.Thread(target=run, daemon=True)
        self.thread.start()
        first.wait(1.5)   # the timed region starts once the first sample is in

    def _start_smi(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-lms", "50"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        # the timed region starts once the first sample is in (at most 1.5 s)
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 1.5 and self.proc.poll() is None:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.02)

    def stop(self, gpu_index=0):
        if self.thread is not None:
            self.stop_evt.set()
            self.thread.join(timeout=5)
            self.thread = None
            self.lib.nvmlShutdown()
            return clock_record(self.samples, "nvml", self.interval_ms)
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        samples = []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9 or f[0] != str(gpu_index):
                continue
            try:
                sm, smax = float(f[1]), float(f[2])
            except ValueError:
                continue
            samples.append((sm, smax, [nm for nm, v in zip(names, f[5:9]) if v.lower().startswith("active")]))
        os.unlink(self.path)
        return clock_record(samples, "nvidia-smi", 50)


def plain_bytes_per_step(cfg):
    """Algorithmic bytes of one plain FP32 step: 352 B per particle (cube keys
    20, sort 48, state permutation 132, cube ranges 4, density 20, force 44,
    integration 84) + 16 per triangle + 32 per edge + 28 per membrane vertex."""
    return 352 * cfg.n + 16 * cfg.ntri + 32 * cfg.nedge + 28 * cfg.ncp


# Per-particle byte counts of the fused step's kernels.  fk_force's share of
# the plain step's algorithmic bytes: the fused force pass (44 B: position,
# velocity, pressure and density read, force written) and the corrector of the
# integration (28 B: VelHalf read, velocity written).
FORCE_ALG_BYTES = 44 + 28
# Bytes of the particle's own records fk_force moves: its position, predicted
# velocity and VelHalf (16 B each) and (1/d, P/d^2) (8 B) read, force and
# velocity (16 B each) written, the list length (4 B) read.  The neighbour
# list entries it streams (4 B each) come on top: the Verlet lists are an
# implementation overhead of the fused step, not algorithmic bytes.
FORCE_STATE_BYTES = 16 * 3 + 8 + 16 * 2 + 4
# Partial sums of the pair tiles per particle, written by the pair pass and
# read back by its finish: 14 directions x 3 floats (force), x 1 (density).
TILE_PARTIAL_BYTES = {"force": 2 * 14 * 12, "density": 2 * 14 * 4}

# Counters from one-kernel ncu captures of fk_force (they are constants of
# the kernel's code, refreshed whenever it changes; the line says which
# capture they come from):
#   python bench.py --small --no-ensemble --cpu-steps 0 --no-plain --no-engine --no-output --no-parity
#       --no-configs --no-variants --steps 3 --warmup 3 --profile-steps 1 --e2e-steps 1   (plain run, exit 0),
#   then ncu --set full --clock-control none -k regex:"fk_(force|density)" -s 6 -c 2 <the same command>
# on the 524,288-particle suspension (warp instructions and FP32 operations
# per particle; skin 0.125 rc, mean list 166.5), and
#   ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum --clock-control none
#       -k regex:"fk_(force|density|build_list|mgather|medge|mgeo|mtri|integrate)" -s 8 -c 8 python bench.py
#       --no-ensemble --cpu-steps 0 --no-plain --no-engine --no-output --no-parity --no-configs --no-variants
#       --steps 4 --warmup 3 --profile-steps 1 --e2e-steps 1
# at full size (DRAM bytes of one launch, one pass).
FORCE_COUNTERS = {
    "kernel_version": "fk_force<1,0,0,1,0>: one thread per particle over its compact list of acting entries, "
                      "pair terms as three coefficient vectors, noise and wall-free forms as template switches",
    "dram_bytes_per_launch_4M": 3.256612864e9 + 0.129022976e9,
    "warp_inst_per_particle": 278141655 / 524288,
    "fp32_flop_per_particle": 4.1227e9 / 524288,
}
# SM schedulers of a GB300 (152 SMs x 4, one warp instruction per cycle
# each) and its FP32 lanes (152 SMs x 128, an FMA counting 2).
GB300_SCHEDULERS = 152 * 4
GB300_FP32_FLOP_PER_CYCLE = 152 * 128 * 2


def rooflines(cfg, ms_per_step, force_ms, dens_ms, mean_nb, hbm, peak_kind, clocks, full_size, tiles=False):
    """The roofline objects of the bench line.

    `roofline`: the whole step against HBM, with the algorithmic bytes of the
    plain FP32 step (plain_bytes_per_step: 352 B per particle + 16 per
    triangle + 32 per edge + 28 per membrane vertex), so that frac =
    particle-steps/s x B_alg / N / the measured HBM bandwidth.
    `roofline_kernels`: fk_force with its share of those bytes (force 44 +
    corrector 28 per particle), and the bytes it actually streams (its own
    records plus 4 B per neighbour-list entry, the lists being overhead);
    fk_density likewise.  `issue_roofline` / `fp32_roofline`: fk_force's
    warp instructions and FP32 operations (ncu counters of its code) per
    second against the GB300's issue and FP32 peaks, the roofs that bind it.
    """
    n = cfg.n
    peak_src = f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"
    b_alg = plain_bytes_per_step(cfg)
    step_gbs = b_alg / (ms_per_step / 1e3) / 1e9
    roof = {
        "kernel": "whole fused step",
        "bound": "hbm",
        "achieved": step_gbs,
        "peak": hbm,
        "unit": "GB/s",
        "frac": step_gbs / hbm,
        "peak_source": peak_src,
        "traffic": None,
        "bytes_per_step": b_alg,
        "formula": f"B_alg = 352 N + 16 N_tri + 32 N_edge + 28 N_vert = 352*{n} + 16*{cfg.ntri} + 32*{cfg.nedge} "
                   f"+ 28*{cfg.ncp} = {b_alg / 1e9:.4f} GB per step; frac = B_alg / (ms_per_step) / peak",
        "note": "algorithmic bytes of the plain FP32 step per unit of work (neighbour state from cache, no lists); "
                "the fused step is bound by instruction issue and gather latency in its pair kernels (issue_roofline)",
    }
    f_alg = FORCE_ALG_BYTES * n
    d_alg = 20 * n
    if tiles:
        # pair tiles: one 4-byte entry per candidate pair (mean_nb / 2 per
        # particle), 14 partial-sum planes written and read back by the finish
        f_streamed = n * (FORCE_STATE_BYTES + TILE_PARTIAL_BYTES["force"] + 4 * mean_nb / 2)
        d_streamed = n * (24 + TILE_PARTIAL_BYTES["density"] + 4 * mean_nb / 2)
        f_note = (f"streamed = {FORCE_STATE_BYTES} B of the particle's records + {TILE_PARTIAL_BYTES['force']} B of "
                  f"partial sums per particle + 4 B per candidate pair ({mean_nb / 2:.1f} per particle)")
        d_note = (f"streamed = 24 + {TILE_PARTIAL_BYTES['density']} B of partial sums per particle + 4 B per "
                  "candidate pair")
    else:
        f_streamed = n * (FORCE_STATE_BYTES + 4 * mean_nb)
        d_streamed = n * (24 + 4 * mean_nb)
        f_note = f"streamed = {FORCE_STATE_BYTES} B per particle + 4 B per list entry (mean list {mean_nb:.1f})"
        d_note = "streamed = 24 B per particle + 4 B per list entry"
    kern = {
        "fk_force": {
            "launch_ms": force_ms, "bound": "hbm", "unit": "GB/s", "peak": hbm, "peak_source": peak_src,
            "alg_bytes_per_launch": f_alg, "achieved": f_alg / (force_ms / 1e3) / 1e9,
            "frac": f_alg / (force_ms / 1e3) / 1e9 / hbm,
            "streamed_bytes_per_launch": f_streamed,
            "streamed_frac": f_streamed / (force_ms / 1e3) / 1e9 / hbm,
            "traffic": FORCE_COUNTERS["dram_bytes_per_launch_4M"] if full_size else None,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch at full size "
                              f"({FORCE_COUNTERS['kernel_version']})",
            "note": f"alg = {FORCE_ALG_BYTES} B per particle (force 44 + corrector 28); {f_note} (overhead)",
        },
        "fk_density": {
            "launch_ms": dens_ms, "bound": "hbm", "unit": "GB/s", "peak": hbm,
            "alg_bytes_per_launch": d_alg, "achieved": d_alg / (dens_ms / 1e3) / 1e9,
            "frac": d_alg / (dens_ms / 1e3) / 1e9 / hbm,
            "streamed_bytes_per_launch": d_streamed,
            "streamed_frac": d_streamed / (dens_ms / 1e3) / 1e9 / hbm,
            "note": f"alg = 20 B per particle (position read, density written); {d_note}",
        },
    }
    mhz = clocks["sm_mhz"] if clocks else 2070.0
    ipp, fpp = FORCE_COUNTERS["warp_inst_per_particle"], FORCE_COUNTERS["fp32_flop_per_particle"]
    issue = {
        "kernel": "fk_force", "bound": "instruction issue", "unit": "warp instructions/s",
        "achieved": ipp * n / (force_ms / 1e3), "peak": GB300_SCHEDULERS * mhz * 1e6,
        "frac": ipp * n / (force_ms / 1e3) / (GB300_SCHEDULERS * mhz * 1e6),
        "note": f"{ipp:.0f} warp instructions per particle (ncu, 524k-particle suspension, "
                f"{FORCE_COUNTERS['kernel_version']}); peak = 608 schedulers x the sampled SM clock",
    }
    fp32 = {
        "kernel": "fk_force", "bound": "FP32 pipe", "unit": "TFLOP/s",
        "achieved": fpp * n / (force_ms / 1e3) / 1e12, "peak": GB300_FP32_FLOP_PER_CYCLE * mhz * 1e6 / 1e12,
        "frac": fpp * n / (force_ms / 1e3) / (GB300_FP32_FLOP_PER_CYCLE * mhz * 1e6),
        "note": f"{fpp:.0f} FP32 operations per particle (FADD + FMUL + 2 FFMA, ncu); peak = 152 SMs x 128 lanes "
                "x 2 x the sampled SM clock",
    }
    return roof, kern, issue, fp32


def measure_plain(cfg, dev, steps, warmup, engine=False):
    """The boundary entry points called in GPUCell's step order, timed with
    CUDA events: with engine=False one kernel per entry point (the
    reference-structured FP32 step, the FP32 denominator); with engine=True
    the fused engine behind them (GPUCELL_ENGINE=fused: each call sequence
    runs as one fused step and writes back every buffer the host reads)."""
    import torch
    from gpucell_gb300 import _lib
    from gpucell_gb300.host import ParticleSystem
    _lib.call("gc_set_engine", 1 if engine else 0)
    ps = ParticleSystem(cfg, device=dev, noise=True)
    for _ in range(warmup):
        ps.update()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    l0 = _lib.launch_count()
    e0.record()
    for _ in range(steps):
        ps.update()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    out = {"ms_per_step": ms, "value": cfg.n / (ms / 1e3), "steps": steps,
           "gpu_launches_per_step": (_lib.launch_count() - l0) / steps, "dtype": "fp32",
           "path": "boundary entry points (gc_cupar_*/gc_cudiv_*), one kernel each" if not engine else
                   "boundary entry points in GPUCell's order with GPUCELL_ENGINE=fused: one fused step per call "
                   "sequence, every host-read buffer written back each step"}
    if engine:
        out["dtype"] = "fp32 pair physics; double-float positions; fp64 membrane sums"
    del ps
    torch.cuda.synchronize()
    _lib.call("gc_set_engine", 0)
    return out


def rank_reducers(world, dev):
    """The barrier and the max over ranks that bracket every timed region
    (identities on one process).  Times are reduced as float64 tensors on
    `dev`: the GPU under NCCL, the CPU under gloo."""
    import torch
    import torch.distributed as dist

    def barrier():
        if world > 1:
            dist.barrier()

    def max_over_ranks(x):
        if world == 1:
            return x
        t = torch.tensor([x], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    return barrier, max_over_ranks


def run_ours(args):
    import numpy as np
    import torch
    import torch.distributed as dist

    from gpucell_gb300 import _lib
    from gpucell_gb300.build import build_library
    from gpucell_gb300.fused import FusedSystem, _ptr

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if rank == 0:
        build_library()
    if world > 1:
        dist.barrier()

    barrier, max_over_ranks = rank_reducers(world, dev)

    if args.rouleaux_run or args.constriction_run:
        if rank == 0:
            print(json.dumps(run_rouleaux(args) if args.rouleaux_run else run_constriction(args)), flush=True)
        if world > 1:
            dist.destroy_process_group()
        return

    if args.ensemble_only:
        ens = run_ensemble(args, dev, rank, world, barrier, max_over_ranks)
        if rank == 0:
            print(json.dumps(ens), flush=True)
        if world > 1:
            dist.destroy_process_group()
        return

    cfg, wdesc = workload(args, rank)
    W = max(args.warmup, 3)
    K = args.steps
    plain = measure_plain(cfg, dev, steps=min(K, 10), warmup=3) if args.plain else None
    engine = measure_plain(cfg, dev, steps=K, warmup=3, engine=True) if args.engine else None

    fs = FusedSystem(cfg, noise=args.noise, skin=args.skin, block=args.block, compact=args.compact,
                     graph=args.graph, tiles=args.tiles)
    fs.step(W, 1)
    tuned = fs.autotune(trial_steps=args.tune_steps) if args.tune else None
    fs.step(2, 1)   # settle (captures the step graph when one is used)
    opts = fs.options()
    torch.cuda.synchronize()
    sampler = ClockSampler()
    if rank == 0:
        sampler.start(local)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    l0 = _lib.launch_count()
    st0 = fs.stats()
    ev0.record()
    fs.step(K, 1)
    ev1.record()
    torch.cuda.synchronize()
    barrier()
    launches = _lib.launch_count() - l0
    t_ms = max_over_ranks(ev0.elapsed_time(ev1))
    clocks = sampler.stop(local) if rank == 0 else None
    st1 = fs.stats()
    diag = fs.diagnostics()
    # per-kernel CUDA-event timing on the launching stream (a separate pass,
    # host-driven, so that the timed steps above run as configured)
    fs.profile(True)
    fs.step(max(1, args.profile_steps), 1)
    prof = fs.profile_read()
    fs.profile(False)
    flags = fs.flags()

    # ---- end to end: host state -> device, one step, results -> host ----
    n = cfg.n
    pin = lambda shape, dt: torch.empty(shape, dtype=dt).pin_memory()
    h = {k: pin((n, 3), torch.float32) for k in ("pos", "vel", "velhalf", "force")}
    h["nthro"] = pin((n, 3), torch.int32)
    h["rho"], h["press"] = pin((n,), torch.float32), pin((n,), torch.float32)
    hc = {}
    if cfg.ncell:
        hc = {"area": pin((cfg.ncell,), torch.float32), "vol": pin((cfg.ncell,), torch.float32),
              "defforce": pin((cfg.ncp, 3), torch.float32), "aggforce": pin((cfg.ncp, 3), torch.float32),
              "trinordir": pin((cfg.ntri, 3), torch.float32), "tricenter": pin((cfg.ntri, 3), torch.float32)}

    def store():
        _lib.call("gc_fused_store", fs.h, *[_ptr(h[k]) for k in ("pos", "vel", "rho", "press", "force", "velhalf",
                                                                 "nthro")], 0)
        if hc:
            _lib.call("gc_fused_store_cells", fs.h, *[_ptr(hc[k]) for k in ("area", "vol", "defforce", "aggforce",
                                                                           "trinordir", "tricenter")],
                      _ptr(None), 0)

    store()
    bi = sum(h[k].numel() * h[k].element_size() for k in ("pos", "vel", "velhalf", "force", "nthro"))
    bo = sum(t.numel() * t.element_size() for t in list(h.values()) + list(hc.values()))
    KE = max(1, args.e2e_steps)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    cell_ptrs = [_ptr(hc.get(k)) for k in ("area", "vol", "defforce", "aggforce", "trinordir", "tricenter")]
    for _ in range(KE):
        _lib.call("gc_fused_load", fs.h, *[_ptr(h[k]) for k in ("pos", "vel", "velhalf", "force", "nthro")], 0)
        # one step, its outputs copied to the host buffers as they become final
        _lib.call("gc_fused_step_store", fs.h, 1,
                  *[_ptr(h[k]) for k in ("pos", "vel", "rho", "press", "force", "velhalf", "nthro")], *cell_ptrs,
                  _ptr(None))
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0)

    out_info = None
    if args.output and rank == 0:
        import shutil
        tmp = tempfile.mkdtemp(prefix="gc_output_")
        try:
            t0 = time.perf_counter()
            fs.write_output(os.path.join(tmp, "Result"), 1, 1e-3, first=True)
            dt = time.perf_counter() - t0
            size = sum(os.path.getsize(os.path.join(r, f)) for r, _, fl in os.walk(tmp) for f in fl)
            out_info = {"seconds": dt, "bytes": size, "threads": os.cpu_count(),
                        "what": "one output step: store, per-cell GPU reductions, FluidCoor, FluidField, CellCoor, "
                                "CellForce, CellNorDir, TF_Cell/Geo_Cell lines (gc_fused_write_output)"}
        finally:
            shutil.rmtree(tmp, ignore_errors=True)

    n_all = n * world
    value = n_all * K / (t_ms / 1e3)
    e2e_value = n_all * KE / e2e_s
    peaks, peak_kind = measured_peaks()
    hbm = float(peaks["hbm_gbs"])
    mean_nb = st1["mean_neighbors"]
    force_ms = prof["force_ms"] / max(prof["steps"], 1)
    dens_ms = prof["density_ms"] / max(prof["steps"], 1)
    roof, roof_kernels, issue_roof, fp32_roof = rooflines(cfg, t_ms / K, force_ms, dens_ms, mean_nb, hbm, peak_kind,
                                                          clocks, full_size=(not args.small and n == 4194304),
                                                          tiles=opts["tiles"])

    fs.close()
    variants = time_variants(cfg, args, min(K, 30)) if args.variants and world == 1 else None
    ens = run_ensemble(args, dev, rank, world, barrier, max_over_ranks) if args.ensemble else None
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    configs = run_config_legs(args) if args.configs and world == 1 else None

    cpu, parity = cpu_leg(cfg, args.cpu_steps if world == 1 else 0, args.parity, args)
    line = {
        "metric": metric_name(n),
        "value": value,
        "unit": "particle-steps/s",
        "n_gpus": world,
        "steps": K,
        "warmup": W,
        "ms_per_step": t_ms / K,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32 pair physics; double-float (fp32 pair) positions; fp64 membrane area/volume sums",
        "data": "synthetic (seeded generator, no dataset)",
        "variant": ("fused step, pair tiles: each pair once per pass, both sides from one evaluation "
                    "(gc_fused_*)") if opts["tiles"] else
                   "fused step: per-particle Verlet lists with skin, fused passes (gc_fused_*)",
        "config": dict(wdesc, particles=n, membrane_vertices=cfg.ncp, triangles=cfg.ntri, edges=cfg.nedge,
                       parallelism=f"replicas x{world}" if world > 1 else "single GPU",
                       l2="working set (>1 GB: state + neighbour lists) is larger than L2; no flush",
                       noise="on" if args.noise else "off", skin=opts["skin"], block=opts["block"],
                       pair_tiles=opts["tiles"], compact_lists=None if opts["tiles"] else opts["compact"],
                       captured_steps=opts["graph"],
                       autotuned=tuned),
        "clocks": clocks,
        "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": bi,
                "d2h_bytes_per_step": bo, "steps": KE,
                "path": "C ABI gc_fused_load -> gc_fused_step_store (outputs copied as they become final), pinned "
                        "host buffers"},
        "gpu_launches": launches,
        "roofline": roof,
        "roofline_kernels": roof_kernels,
        "issue_roofline": issue_roof,
        "fp32_roofline": fp32_roof,
        "kernels_ms_per_step": {"fk_force": force_ms, "fk_density": dens_ms},
        "output_step": out_info,
        "diagnostics_fp64": {"momentum": [float(x) for x in diag["momentum"]],
                             "kinetic_energy": diag["kinetic_energy"], "kT": diag["temperature"],
                             "max_speed": diag["max_speed"], "mean_fluid_density": diag["mean_fluid_density"],
                             "note": "after the timed steps, reduced on the GPU in FP64 (gc_ensemble_diagnostics)"},
        "parity": parity,
        "lists": {"rebuilds_in_timed_steps": st1["rebuilds"] - st0["rebuilds"], "mean_neighbors": mean_nb,
                  "max_length": st1["max_neighbors"], "capacity": st1["capacity"]},
        "device_flags": flags,
    }
    if plain:
        plain["speedup_of_fused"] = plain["ms_per_step"] / (t_ms / K)
        line["plain_fp32"] = plain
    if engine:
        if plain:
            engine["speedup_over_plain"] = plain["ms_per_step"] / engine["ms_per_step"]
        line["engine_fused"] = engine
    if variants:
        ref_ms = variants["default"]["ms_per_step"]
        for v in variants.values():
            v["slowdown_vs_default"] = v["ms_per_step"] / ref_ms   # the same window of steps
        line["variants"] = variants
    if ens:
        line["ensemble"] = ens
    if configs:
        line["configs"] = configs
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


ENS_METRIC = "particle-steps/s on a 64-suspension ensemble (8k-200k particles, 0-16 cells of 642 vertices)"


def run_rouleaux(args):
    """Aggregation under shear: 64 cells of 2562 vertices at random positions
    and orientations in Couette flow (walls moving at -+U, Morse aggregation
    De = 3e-3, beta = 1.5, r0 = 0.3, cut-off 2.5, thermal noise on at
    k_B T = `rouleaux_temp`), the same
    initial state at each shear rate; every `rouleaux_every` steps the
    rouleaux are found on the GPU (cells in contact: a vertex pair closer than
    `rouleaux_contact`).  Steps are timed with CUDA events, the rouleau
    searches apart."""
    import dataclasses

    import numpy as np
    import torch
    from gpucell_gb300 import generator
    from gpucell_gb300.fused import FusedSystem

    runs = []
    S, E = max(1, args.rouleaux_steps), max(1, args.rouleaux_every)
    phys = dataclasses.replace(generator.Physics(ext_force=0.0, sur_energy=3.0e-3, sca_fac=1.5, zero_len=0.3,
                                                 max_cut=2.5), temp=args.rouleaux_temp)
    for rate in [float(x) for x in args.shear_rates.split(",") if x]:
        cfg = generator.sheared_suspension(shear_rate=rate, phys=phys)
        fs = FusedSystem(cfg, noise=args.noise, skin=0.1, compact=True, graph=args.graph)
        fs.step(3, 1)
        torch.cuda.synchronize()
        series, step_ms, search_ms = [], 0.0, []
        done = 0

        def sample():
            t0 = time.perf_counter()
            _, size = fs.rouleaux(args.rouleaux_contact)
            search_ms.append(1e3 * (time.perf_counter() - t0))
            series.append([done, int(size.size), int(size.max()), float(size.mean())])

        sample()
        r0 = fs.stats()["rebuilds"]
        sampler = ClockSampler()
        sampler.start()
        while done < S:
            k = min(E, S - done)
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record()
            fs.step(k, 0)
            ev1.record()
            torch.cuda.synchronize()
            step_ms += ev0.elapsed_time(ev1)
            done += k
            sample()
        clocks = sampler.stop()
        st = fs.stats()
        flags = fs.flags()
        fs.close()
        runs.append({"shear_rate": rate, "wall_speed": cfg.meta["wall_speed"], "clocks": clocks,
                     "list_rebuilds": st["rebuilds"] - r0, "max_list": st["max_neighbors"],
                     "strain": rate * S * cfg.phys.dt, "ms_per_step": step_ms / S,
                     "particle_steps_per_s": cfg.n * S / (step_ms / 1e3), "rouleau_search_ms": float(np.median(search_ms)),
                     "device_flags": flags,
                     "series_columns": ["step", "rouleaux", "largest", "mean_cells"], "series": series})
    return {"workload": "sheared_suspension", "particles": cfg.n, "fluid": cfg.n_fluid, "walls": cfg.n_b2,
            "cells": cfg.ncell, "vertices_per_cell": int(cfg.npar[0]), "steps": S, "dt": cfg.phys.dt,
            "contact": args.rouleaux_contact, "noise": "on" if args.noise else "off", "kT": cfg.phys.temp,
            "captured_steps": bool(args.graph),
            "morse": {"De": cfg.phys.sur_energy, "beta": cfg.phys.sca_fac, "r0": cfg.phys.zero_len,
                      "cutoff": cfg.phys.max_cut},
            "data": "synthetic (seeded generator, no dataset)", "runs": runs}


def cell_geometry_fp64(cfg, pos, nthro):
    """Area and volume of every cell in FP64 on the host, from the stored FP32
    positions unwrapped by their crossing counts (x + n L on periodic axes):
    triangle areas |(b - a) x (c - a)| / 2 and, by the divergence theorem,
    volumes a . (b x c) / 6, summed over each cell's triangles."""
    import numpy as np
    L = (cfg.bbox[1::2].astype(np.float64) - cfg.bbox[0::2].astype(np.float64))
    L = L * np.array([(cfg.pmask >> k) & 1 for k in range(3)], np.float64)
    cs = cfg.n_cell_start
    m = pos[cs:].astype(np.float64) + nthro[cs:].astype(np.float64) * L
    t = cfg.tri.astype(np.int64) - 1
    a, b, c = m[t[:, 0]], m[t[:, 1]], m[t[:, 2]]
    area_t = 0.5 * np.linalg.norm(np.cross(b - a, c - a), axis=1)
    vol_t = np.einsum("ij,ij->i", a, np.cross(b, c)) / 6.0
    first = cfg.betri[:, 0].astype(np.int64)
    return np.add.reduceat(area_t, first), np.add.reduceat(vol_t, first)


def run_constriction(args):
    """Complex geometry: 100 cells of 642 vertices at random positions and
    orientations in a channel with a 2:1 constriction of frozen wall
    particles (1,951,322 particles), driven by the body force.  Every
    `check_every` steps the GPU's FP64 per-cell area and volume are checked
    against an FP64 host evaluation from the stored positions, and their
    drift from the values after three warm-up steps is recorded.  Steps are
    timed with CUDA events, the checks apart."""
    import numpy as np
    import torch
    from gpucell_gb300 import generator
    from gpucell_gb300.fused import FusedSystem

    cfg = generator.constriction(nx=280, ny=96, nz=72, ncells=100, subdiv=3, layout="random")
    fs = FusedSystem(cfg, noise=args.noise, skin=0.075, compact=True, graph=args.graph)
    S, E = max(1, args.constriction_steps), max(1, args.check_every)
    fs.step(3, 1)   # warm-up (the kernels of a walled system load on their first launch)
    torch.cuda.synchronize()
    g = fs.fetch()
    a0, v0 = g["Area64"].copy(), g["Vol64"].copy()
    checks, step_ms, done = [], 0.0, 0

    def check():
        g = fs.fetch()
        ha, hv = cell_geometry_fp64(cfg, g["pos"], g["nthro"])
        checks.append([done, float(np.abs(g["Area64"] / ha - 1).max()), float(np.abs(g["Vol64"] / hv - 1).max()),
                       float(np.abs(g["Area64"] / a0 - 1).max()), float(np.abs(g["Vol64"] / v0 - 1).max())])

    check()
    r0 = fs.stats()["rebuilds"]
    sampler = ClockSampler()
    sampler.start()
    while done < S:
        k = min(E, S - done)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        fs.step(k, 1)
        ev1.record()
        torch.cuda.synchronize()
        step_ms += ev0.elapsed_time(ev1)
        done += k
        check()
    clocks = sampler.stop()
    st = fs.stats()
    flags = fs.flags()
    fs.close()
    arr = np.array(checks)
    return {"workload": "constriction", "particles": cfg.n, "fluid": cfg.n_fluid, "walls": cfg.n_b1 + cfg.n_b2,
            "cells": cfg.ncell, "vertices_per_cell": int(cfg.npar[0]), "steps": S, "dt": cfg.phys.dt,
            "noise": "on" if args.noise else "off", "captured_steps": bool(args.graph),
            "ms_per_step": step_ms / S, "particle_steps_per_s": cfg.n * S / (step_ms / 1e3),
            "max_area_error_vs_fp64_host": float(arr[:, 1].max()),
            "max_volume_error_vs_fp64_host": float(arr[:, 2].max()),
            "checks_columns": ["step", "area_error", "volume_error", "area_drift", "volume_drift"],
            "checks": checks, "list_rebuilds": st["rebuilds"] - r0, "max_list": st["max_neighbors"],
            "device_flags": flags, "clocks": clocks, "data": "synthetic (seeded generator, no dataset)"}


def run_ensemble(args, dev, rank, world, barrier, max_over_ranks):
    """Independent suspensions of uneven size stepped together (one ensemble
    per GPU, systems shared out by LPT over ranks), against the same systems
    run one after the other on the FP32 boundary path and on the fused step
    alone.  Returns the summary on rank 0, None elsewhere."""
    import torch
    from gpucell_gb300 import _lib, generator, shard
    from gpucell_gb300.fused import Ensemble, FusedSystem
    from gpucell_gb300.host import ParticleSystem

    cfgs = generator.ensemble_suite(nsys=args.ens_systems, seed=2024)
    mine = shard.shard_for_rank([c.n for c in cfgs], rank, world)
    sub = [cfgs[i] for i in mine]
    K = max(1, args.ens_steps)
    ens = Ensemble(sub, noise=args.noise, skin=0.1, block=128, compact=True, graph=True)
    ens.step(max(args.warmup, 3), 1)
    tuned = ens.autotune(trial_steps=10)
    ens.step(2, 1)
    opts = ens.options()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    l0 = _lib.launch_count()
    r0 = ens.stats()["rebuilds"]
    ev0.record()
    ens.step(K, 1)
    ev1.record()
    torch.cuda.synchronize()
    barrier()
    launches = _lib.launch_count() - l0
    t_ms = max_over_ranks(ev0.elapsed_time(ev1))
    est = ens.stats()
    rebuilds = est["rebuilds"] - r0
    flags = ens.flags()
    ens.close()
    if rank != 0:
        return None
    n_all = sum(c.n for c in cfgs)
    out = {"metric": ENS_METRIC, "value": n_all * K / (t_ms / 1e3), "unit": "particle-steps/s",
           "ms_per_step": t_ms / K, "steps": K, "systems": len(cfgs), "particles": n_all,
           "membrane_vertices": sum(c.ncp for c in cfgs), "cells": sum(c.ncell for c in cfgs),
           "particles_min": min(c.n for c in cfgs), "particles_max": max(c.n for c in cfgs),
           "options": opts, "autotuned": tuned, "gpu_launches": launches,
           "lists": {"rebuilds_in_timed_steps": rebuilds, "mean_length": est["mean_neighbors"],
                     "max_length": est["max_neighbors"], "capacity": est["capacity"]},
           "device_flags": flags, "data": "synthetic (generator.ensemble_suite, seed 2024)",
           "sharding": f"LPT over {world} ranks, {len(sub)} systems on rank 0" if world > 1 else "one GPU"}
    if world > 1:
        return out
    # the same systems one after the other: FP32 boundary path, fused step
    seq_plain_ms = seq_fused_ms = 0.0
    ps_steps, fs_steps = max(1, args.ens_seq_steps), K
    seq_launches = 0
    for c in sub:
        ps = ParticleSystem(c, device=dev, noise=args.noise)
        for _ in range(3):   # warm-up
            ps.update()
        torch.cuda.synchronize()
        l1 = _lib.launch_count()
        ev0.record()
        for _ in range(ps_steps):
            ps.update()
        ev1.record()
        torch.cuda.synchronize()
        seq_plain_ms += ev0.elapsed_time(ev1)
        seq_launches += _lib.launch_count() - l1
        del ps
        fs = FusedSystem(c, noise=args.noise, skin=0.1, block=128, compact=True)
        fs.step(3, 1)
        torch.cuda.synchronize()
        ev0.record()
        fs.step(fs_steps, 1)
        ev1.record()
        torch.cuda.synchronize()
        seq_fused_ms += ev0.elapsed_time(ev1)
        fs.close()
    plain_v = n_all * ps_steps / (seq_plain_ms / 1e3)
    fused_v = n_all * fs_steps / (seq_fused_ms / 1e3)
    out["sequential_plain_fp32"] = {"value": plain_v, "unit": "particle-steps/s",
                                    "ms_per_step_all_systems": seq_plain_ms / ps_steps, "steps_each": ps_steps,
                                    "gpu_launches_per_step": seq_launches / ps_steps,
                                    "path": "the systems one after the other, boundary entry points, FP32"}
    out["sequential_fused"] = {"value": fused_v, "unit": "particle-steps/s",
                               "ms_per_step_all_systems": seq_fused_ms / fs_steps, "steps_each": fs_steps,
                               "path": "the systems one after the other, fused step, host-driven"}
    out["speedup_vs_sequential_plain_fp32"] = out["value"] / plain_v
    out["speedup_vs_sequential_fused"] = out["value"] / fused_v
    return out


def cpu_leg(cfg, cpu_steps, parity, args):
    """The FP64 CPU oracle's leg of the bench (rank 0, after the timed GPU
    work).  `cpu_baseline` times `cpu_steps` full oracle steps of the
    workload on all host cores after one warm-up step, and a one-core sample.
    With `parity`, the same oracle run doubles as the checker of the
    workload itself: after its first five steps (the warm-up and four timed
    ones, the clock stopped while it compares) it is compared with five
    fused steps of the GPU from the same state (noise on, the same Philox
    pair noise); a second oracle state evaluates the forces once on the
    set-up positions (a vanishing time step, noise off) against the GPU's,
    particle by particle; and a small walled channel is stepped 100 times by
    both.  The oracle is used nowhere else here."""
    from gpucell_gb300.build import build_oracle
    if cpu_steps <= 0 and not parity:
        return None, None
    build_oracle()
    par = {}
    if parity:
        par = force_parity(cfg)
    cpu, traj = cpu_baseline(cfg, cpu_steps, compare_after=5 if parity else 0)
    if parity:
        par["trajectory"] = traj
        par["channel"] = parity_check(100)
        par["precision_variants"] = precision_parity()
        par["workload"] = f"{cfg.n}-particle RBC suspension ({cfg.ncell} cells of {int(cfg.npar[0])} vertices)"
        par["reference"] = "FP64 CPU oracle (oracle/oracle.c)"
    return (cpu if cpu_steps > 0 else None), (par or None)


def precision_parity(steps=300):
    """The precision variants against the FP64 oracle: the largest position
    error of a walled channel with a cell after `steps` steps (noise off)
    with double-float and with plain FP32 positions; and the per-particle
    force error of one force evaluation on a stepped periodic suspension with
    FP32 and with FP16-packed neighbour velocities."""
    import dataclasses

    import numpy as np
    from gpucell_gb300 import generator
    from gpucell_gb300.fused import FusedSystem
    from oracle.binding import Oracle, force_error_stats
    cfg = generator.small_channel()
    o = Oracle(cfg, noise=False, nthreads=os.cpu_count() or 1)
    o.setup()
    for _ in range(steps):
        o.step()
    drift = {}
    for name, fp32 in (("double_float", False), ("fp32", True)):
        fs = FusedSystem(cfg, noise=False, fp32_positions=fp32)
        fs.step(steps, 1)
        d = fs.fetch()["pos"].astype(np.float64) - o.pos
        fs.close()
        for a in range(3):
            if (cfg.pmask >> a) & 1:
                L = float(cfg.bbox[2 * a + 1] - cfg.bbox[2 * a])
                d[:, a] -= L * np.rint(d[:, a] / L)
        drift[name] = float(np.abs(d).max())
    sus = generator.suspension(nx=32, ny=24, nz=24, ncells=2, subdiv=2, hematocrit=0.12, seed=6)
    warm = FusedSystem(sus, noise=True)
    warm.step(20, 1)
    s = warm.fetch()
    warm.close()
    c0 = dataclasses.replace(sus, phys=dataclasses.replace(sus.phys, dt=1e-20))
    o = Oracle(c0, noise=False, nthreads=os.cpu_count() or 1)
    o.setup()
    o.set(pos=s["pos"], vel=s["vel"], velhalf=s["velhalf"], force=s["force"], nthro=s["nthro"])
    o.step()
    mov = slice(sus.n_b1 + sus.n_b2, sus.n)
    scale = o.force_scale()[mov]
    ferr = {}
    for name, half in (("fp32", False), ("fp16", True)):
        fs = FusedSystem(c0, noise=False, half_velocity=half)
        fs.load(s["pos"], s["vel"], s["velhalf"], s["force"], s["nthro"])
        fs.step(1, 1)
        g = fs.fetch()
        fs.close()
        st = force_error_stats(g["force"][mov], o.force[mov], scale)
        ferr[name] = {k: st[k] for k in ("median_rel", "p99_rel", "max_rel", "frac_within_rtol", "worst_ratio")}
    return {"position_error_after_steps": drift, "steps": steps,
            "position_workload": f"walled channel, {cfg.n} particles, one {cfg.ncp}-vertex cell, noise off",
            "neighbour_velocity_force_error": ferr,
            "force_workload": f"periodic suspension, {sus.n} particles, {sus.ncell} cells, velocities of 20 noisy "
                              "steps, one force evaluation"}


def force_parity(cfg):
    """Forces of one fused step on the set-up positions (time step 1e-20, so
    the positions stay; noise off, since the random force grows as dt^-1/2)
    against the FP64 oracle's, per particle: |dF_i| against 1e-5 |F_i| +
    16 u S_i (u = 2^-24, S_i the sum of the magnitudes of the terms F_i adds
    up), with the median, 99th percentile and largest relative errors."""
    import dataclasses

    from gpucell_gb300.fused import FusedSystem
    from oracle.binding import Oracle, force_error_stats
    c0 = dataclasses.replace(cfg, phys=dataclasses.replace(cfg.phys, dt=1e-20))
    o = Oracle(c0, noise=False, nthreads=os.cpu_count() or 1)
    o.setup()
    o.step()
    scale = o.force_scale()
    fs = FusedSystem(c0, noise=False)
    fs.step(1, 1)
    g = fs.fetch()
    fs.close()
    mov = slice(cfg.n_b1 + cfg.n_b2, cfg.n)
    cs = cfg.n_cell_start - (cfg.n_b1 + cfg.n_b2)
    out = {"force_evaluation": {}, "force_given_gpu_density": {}}
    parts = (("all", slice(None)), ("fluid", slice(0, cs)), ("membrane", slice(cs, None)))
    for name, sl in parts:
        out["force_evaluation"][name] = force_error_stats(g["force"][mov][sl], o.force[mov][sl], scale[mov][sl])
    o.forces_from_density(g["rho"], g["press"])
    scale = o.force_scale(31)
    for name, sl in parts:
        out["force_given_gpu_density"][name] = force_error_stats(g["force"][mov][sl], o.force[mov][sl],
                                                                 scale[mov][sl])
    out["force_evaluation"]["what"] = ("one force evaluation on identical positions, noise off, against the oracle's "
                                       "own FP64 densities: per particle |dF_i| <= 1e-5 |F_i| + 16 u S_i, the pressure "
                                       "term counted at c^2 rho in S_i (worst_ratio <= 1 passes)")
    out["force_given_gpu_density"]["what"] = ("the same forces against the oracle's FP64 forces from the GPU's FP32 "
                                              "densities and pressures, the pressure term counted at |P| in S_i")
    del o
    return out


def parity_check(steps=100):
    """The fused step against the FP64 oracle on a walled channel with one
    red cell (Bound1 and Bound2 walls, 5.9k particles, noise off): largest
    position error, velocity-profile error (8 bins across the channel,
    relative to the largest bin velocity) and membrane area/volume errors
    after `steps` steps."""
    import numpy as np
    from gpucell_gb300 import generator
    from gpucell_gb300.fused import FusedSystem
    from oracle.binding import Oracle
    cfg = generator.small_channel()
    fs = FusedSystem(cfg, noise=False)
    o = Oracle(cfg, noise=False, nthreads=os.cpu_count() or 1)
    o.setup()
    fs.step(steps, 1)
    for _ in range(steps):
        o.step()
    g = fs.fetch()
    fs.close()
    fl = slice(cfg.n_b1 + cfg.n_b2, cfg.n_cell_start)
    lo, hi = float(cfg.bbox[2]), float(cfg.bbox[3])

    def profile(pos, vel):
        b = np.clip(((pos[fl, 1] - lo) / (hi - lo) * 8).astype(int), 0, 7)
        return np.array([vel[fl, 0][b == k].mean() for k in range(8)])

    pg, po = profile(g["pos"].astype(np.float64), g["vel"].astype(np.float64)), profile(o.pos, o.vel)
    return {"workload": f"walled channel, {cfg.n} particles, one {cfg.ncp}-vertex cell, noise off",
            "steps": steps,
            "max_position_error": float(np.abs(g["pos"] - o.pos).max()),
            "velocity_profile_error": float(np.abs(pg - po).max() / np.abs(po).max()),
            "area_error": float(abs(g["Area64"][0] / o.area[0] - 1)),
            "volume_error": float(abs(g["Vol64"][0] / o.vol[0] - 1))}


def cpu_baseline(cfg, steps, compare_after=0):
    """FP64 CPU restatement of the method on all host cores, on `steps` full
    steps of the same workload after one warm-up step.  With
    `compare_after` = k, the oracle's state after its first k steps is
    compared with k fused GPU steps from the same set-up (outside the timed
    spans); returns (baseline, comparison)."""
    import numpy as np
    from oracle.binding import Oracle
    threads = os.cpu_count() or 1
    o = Oracle(cfg, noise=True, nthreads=threads)
    o.setup()
    o.step()   # warm-up (page-in, thread start-up)
    done, dt, traj = 1, 0.0, None
    while done - 1 < steps or (compare_after and traj is None):
        if compare_after and done == compare_after and traj is None:
            traj = trajectory_parity(cfg, o, compare_after)
            continue
        t0 = time.perf_counter()
        o.step()
        dt += time.perf_counter() - t0
        done += 1
    timed = done - 1
    del o
    # one core, on a bounded sample: one step of a 1/16-size suspension with
    # cells of the same size at about the same hematocrit (262,144
    # particles, 12 cells)
    from gpucell_gb300 import generator
    small = generator.suspension(nx=64, ny=64, nz=64, ncells=12, seed=7, diameter=cell_diameter(cfg))
    o1 = Oracle(small, noise=True, nthreads=1)
    o1.setup()
    t1 = time.perf_counter()
    o1.step()
    dt1 = time.perf_counter() - t1
    base = {"value": cfg.n * timed / dt, "unit": "particle-steps/s", "cores": threads, "kind": "port",
            "steps": timed,
            "sample": f"{timed} full steps of the {cfg.n}-particle workload after one warm-up step, FP64, OpenMP",
            "cpu_model": cpu_model(),
            "one_core": {"value": small.n / dt1, "unit": "particle-steps/s",
                         "sample": f"one step of a {small.n}-particle suspension ({small.ncell} cells of "
                                   f"{int(small.npar[0])} vertices), FP64, 1 thread"}}
    _ = np
    return base, traj


def trajectory_parity(cfg, o, k):
    """k fused GPU steps (noise on) from the set-up against the oracle `o`
    after its first k steps: largest position error (minimum image), largest
    velocity error relative to the largest speed component, and the largest
    per-cell relative area and volume errors (FP64 on both sides)."""
    import numpy as np
    from gpucell_gb300.fused import FusedSystem
    fs = FusedSystem(cfg, noise=True, skin=0.075)
    fs.step(k, 1)
    g = fs.fetch()
    fs.close()
    d = g["pos"].astype(np.float64) - o.pos
    for a in range(3):
        if (cfg.pmask >> a) & 1:
            L = float(cfg.bbox[2 * a + 1] - cfg.bbox[2 * a])
            d[:, a] -= L * np.rint(d[:, a] / L)
    vs = float(np.abs(o.vel).max())
    out = {"steps": k, "noise": "on",
           "max_position_error": float(np.abs(d).max()),
           "max_velocity_error_rel": float(np.abs(g["vel"] - o.vel).max() / vs), "max_speed_component": vs}
    if cfg.ncell:
        out["max_area_error"] = float(np.abs(g["Area64"] / o.area - 1).max())
        out["max_volume_error"] = float(np.abs(g["Vol64"] / o.vol - 1).max())
    return out


def time_variants(cfg, args, steps):
    """The same workload, timed like the headline step (CUDA events on the
    library's stream, after 5 warm-up steps), as configured (`default`: the
    same window of steps for every entry) and with one setting changed:
    plain FP32 positions instead of double-float ones (the precision A/B of
    the step: same passes, same lists), FP16-packed neighbour velocities in
    the force gathers (an experiment), and the pair tiles (each pair
    evaluated once, instead of per-particle lists)."""
    import torch
    from gpucell_gb300.fused import FusedSystem
    out = {}
    for name, kw in (("default", {}), ("fp32_positions", dict(fp32_positions=True)),
                     ("half_velocity", dict(half_velocity=True)), ("pair_tiles", dict(tiles=True))):
        fs = FusedSystem(cfg, noise=args.noise, skin=args.skin, block=args.block, compact=args.compact, **kw)
        fs.step(5, 1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fs.step(steps, 1)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        fs.profile(True)
        fs.step(2, 1)
        prof = fs.profile_read()
        fs.profile(False)
        o = fs.options()
        out[name] = {"ms_per_step": ms, "value": cfg.n / (ms / 1e3), "steps": steps, "device_flags": fs.flags(),
                     "force_ms": prof["force_ms"] / max(prof["steps"], 1),
                     "density_ms": prof["density_ms"] / max(prof["steps"], 1),
                     "tiles": o["tiles"], "fp32_positions": o["fp32_positions"], "half_velocity": o["half_velocity"]}
        fs.close()
    return out


def run_config_legs(args):
    """Short legs of the other configurations, so that every bench line
    carries them: the sheared suspension with Morse aggregation (cfg3) at
    the three shear rates, and the 2:1 constriction (cfg4) with its FP64
    area/volume check, `config_steps` steps each."""
    import copy
    a = copy.copy(args)
    a.rouleaux_steps = a.constriction_steps = max(1, args.config_steps)
    a.rouleaux_every = a.check_every = max(1, args.config_steps // 2)
    out = {"sheared_suspension": run_rouleaux(a), "constriction": run_constriction(a)}
    for leg in out["sheared_suspension"]["runs"]:
        leg.pop("series_columns", None)
    return out


def cell_diameter(cfg):
    """Diameter of the first cell of a configuration (its extent), or None."""
    import numpy as np
    if not cfg.ncell:
        return None
    m = cfg.coor[cfg.n_cell_start:cfg.n_cell_start + int(cfg.npar[0])].astype(np.float64)
    return float(np.ptp(m, axis=0).max())


def cpu_model():
    """The host CPU's model name (or architecture) and logical core count."""
    import platform
    name = None
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                k, _, v = line.partition(":")
                if k.strip() in ("model name", "Model", "CPU part") and v.strip():
                    name = v.strip()
                    break
    except OSError:
        pass
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=5).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                name = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return f"{name or platform.machine()}, {os.cpu_count()} logical cores"


def run_reference(args):
    """The CPU restatement of the method as the reference arm (the reference's
    own GPU kernels are not available; it has no CPU path)."""
    import numpy as np  # noqa: F401

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from gpucell_gb300.build import build_oracle
    from oracle.binding import Oracle
    build_oracle()
    cfg, wdesc = workload(args, 0)
    threads = os.cpu_count() or 1
    o = Oracle(cfg, noise=True, nthreads=threads)
    o.setup()
    warm = 3   # warm-up steps (page-in, thread start-up), as for the GPU arm
    for _ in range(warm):
        o.step()
    steps = max(1, min(args.steps, args.ref_steps_cap))
    t0 = time.perf_counter()
    for _ in range(steps):
        o.step()
    dt = time.perf_counter() - t0
    value = cfg.n * steps / dt
    line = {
        "impl": "reference",
        "metric": metric_name(cfg.n),
        "value": value,
        "unit": "particle-steps/s",
        "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": steps,
        "warmup": warm,
        "ms_per_step": dt / steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp64",
        "data": "synthetic (seeded generator, no dataset)",
        "config": dict(wdesc, particles=cfg.n),
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{steps} full step(s) of the {cfg.n}-particle workload ({args.steps} requested, "
                                   f"capped at {args.ref_steps_cap}), FP64, OpenMP"},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "GPUCell's GPU kernels are not in the reference and it has no CPU path; this arm is the FP64 "
                "CPU restatement of the method (oracle/oracle.c)",
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
