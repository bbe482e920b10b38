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
    ap.add_argument("--skin", type=float, default=0.075)
    ap.add_argument("--block", type=int, default=128)
    ap.add_argument("--no-compact", dest="compact", action="store_false",
                    help="force pass iterates the skin lists instead of the per-step compact lists")
    ap.add_argument("--no-plain", dest="plain", action="store_false", help="skip the FP32 boundary-path timing")
    ap.add_argument("--no-engine", dest="engine", action="store_false",
                    help="skip the boundary entry points with the fused engine behind them")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-steps", type=int, default=1)
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
                    help="skip the parity check against the FP64 oracle on a small channel")
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


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
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
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9 or f[0] != str(gpu_index):
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons)}


def plain_bytes_per_step(cfg):
    """Algorithmic bytes of one plain FP32 step: 352 B per particle (cube keys
    20, sort 48, state permutation 132, cube ranges 4, density 20, force 44,
    integration 84) + 16 per triangle + 32 per edge + 28 per membrane vertex."""
    return 352 * cfg.n + 16 * cfg.ntri + 32 * cfg.nedge + 28 * cfg.ncp


# Dominant kernel of the fused step: fk_force.  Algorithmic bytes per
# particle: its own position, predicted velocity, VelHalf (16 B each) and
# (1/d, P/d^2) (8 B) read, force and velocity (16 B each) written, the list
# length (4 B) and its neighbour-list entries (4 B each) read.
FORCE_STATE_BYTES = 16 * 3 + 8 + 16 * 2 + 4
# DRAM bytes (read + write) of one fk_force launch on the 4.2M-particle
# suspension, from ncu at full size (profiles/fused_step_rbc_suspension_4M_launches.md):
# 2.845e9 read + 0.128e9 written, with 143.6 list entries per particle.
FORCE_TRAFFIC_4M = 2.845227264e9 + 0.127872512e9
# Warp instructions fk_force issues per particle (ncu smsp__inst_executed.sum
# of one launch on the 524,288-particle suspension / particles, mean list
# 143.7; profiles/fk_force_fk_density_rbc_suspension_524k.md), and the SM
# schedulers of a GB300 (152 SMs x 4), each issuing one warp instruction
# per cycle.
FORCE_WARP_INST_PER_PARTICLE = 348382172 / 524288
GB300_SCHEDULERS = 152 * 4
# FP32 operations of fk_force per particle (FADD + FMUL + 2 FFMA, thread
# level) from the same ncu capture: 5.224e9 over 524,288 particles; the
# FP32 peak is 152 SMs x 128 lanes x 2 (FMA) per cycle.
FORCE_FP32_FLOP_PER_PARTICLE = 5.224e9 / 524288   # 9963 per particle
GB300_FP32_FLOP_PER_CYCLE = 152 * 128 * 2


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
                     graph=args.graph)
    fs.step(W, 1)
    tuned = fs.autotune(trial_steps=args.tune_steps) if args.tune else None
    fs.step(2, 1)   # settle (captures the step graph when one is used)
    opts = fs.options()
    torch.cuda.synchronize()
    sampler = ClockSampler()
    if rank == 0:
        sampler.start()
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
    for _ in range(KE):
        _lib.call("gc_fused_load", fs.h, *[_ptr(h[k]) for k in ("pos", "vel", "velhalf", "force", "nthro")], 0)
        fs.step(1, 1)
        store()
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
    force_bytes = n * (FORCE_STATE_BYTES + 4 * mean_nb)
    achieved = force_bytes / (force_ms / 1e3) / 1e9

    fs.close()
    ens = run_ensemble(args, dev, rank, world, barrier, max_over_ranks) if args.ensemble else None
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return

    cpu, parity = cpu_leg(cfg, args.cpu_steps if world == 1 else 0, 100 if args.parity else 0)
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
        "variant": "fused step: Verlet lists with skin, fused passes (gc_fused_*)",
        "config": dict(wdesc, particles=n, membrane_vertices=cfg.ncp, triangles=cfg.ntri, edges=cfg.nedge,
                       parallelism=f"replicas x{world}" if world > 1 else "single GPU",
                       l2="working set (>1 GB: state + neighbour lists) is larger than L2; no flush",
                       noise="on" if args.noise else "off", skin=opts["skin"], block=opts["block"],
                       compact_lists=opts["compact"], captured_steps=opts["graph"],
                       autotuned=tuned),
        "clocks": clocks,
        "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": bi,
                "d2h_bytes_per_step": bo, "steps": KE,
                "path": "C ABI gc_fused_load -> gc_fused_step -> gc_fused_store(_cells), pinned host buffers"},
        "gpu_launches": launches,
        "roofline": {
            "kernel": "fk_force (SDPD + repulsion + body force + membrane add + corrector)",
            "bound": "hbm",
            "achieved": achieved,
            "peak": hbm,
            "unit": "GB/s",
            "frac": achieved / hbm,
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
            "traffic": FORCE_TRAFFIC_4M if (not args.small and n == 4194304) else None,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one fk_force launch, full size",
            "bytes_per_launch": force_bytes,
            "launch_ms": force_ms,
            "note": f"bytes = {FORCE_STATE_BYTES} per particle + 4 per list entry (mean list {mean_nb:.1f}); "
                    "the pair physics is FP32-issue bound",
        },
        "issue_roofline": {
            "kernel": "fk_force",
            "bound": "instruction issue",
            "achieved": FORCE_WARP_INST_PER_PARTICLE * n / (force_ms / 1e3),
            "peak": GB300_SCHEDULERS * (clocks["sm_mhz"] if clocks else 2070.0) * 1e6,
            "unit": "warp instructions/s",
            "frac": FORCE_WARP_INST_PER_PARTICLE * n / (force_ms / 1e3)
                    / (GB300_SCHEDULERS * (clocks["sm_mhz"] if clocks else 2070.0) * 1e6),
            "note": "instructions per particle from ncu on the 524k-particle suspension; peak = 608 schedulers x "
                    "the sampled SM clock x 1 warp instruction per cycle",
        },
        "fp32_roofline": {
            "kernel": "fk_force",
            "bound": "FP32 pipe",
            "achieved": FORCE_FP32_FLOP_PER_PARTICLE * n / (force_ms / 1e3) / 1e12,
            "peak": GB300_FP32_FLOP_PER_CYCLE * (clocks["sm_mhz"] if clocks else 2070.0) * 1e6 / 1e12,
            "unit": "TFLOP/s",
            "frac": FORCE_FP32_FLOP_PER_PARTICLE * n / (force_ms / 1e3)
                    / (GB300_FP32_FLOP_PER_CYCLE * (clocks["sm_mhz"] if clocks else 2070.0) * 1e6),
            "note": "FP32 operations per particle (FADD + FMUL + 2 FFMA) from ncu on the 524k-particle suspension, "
                    "~88 per acting pair; peak = 152 SMs x 128 lanes x 2 x the sampled SM clock",
        },
        "kernels_ms_per_step": {"fk_force": force_ms, "fk_density": dens_ms},
        "output_step": out_info,
        "diagnostics_fp64": {"momentum": [float(x) for x in diag["momentum"]],
                             "kinetic_energy": diag["kinetic_energy"], "kT": diag["temperature"],
                             "max_speed": diag["max_speed"], "mean_fluid_density": diag["mean_fluid_density"],
                             "note": "after the timed steps, reduced on the GPU in FP64 (gc_ensemble_diagnostics)"},
        "parity": parity,
        "lists": {"rebuilds_in_timed_steps": st1["rebuilds"] - st0["rebuilds"], "mean_length": mean_nb,
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
    if ens:
        line["ensemble"] = ens
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
    drift from the set-up values is recorded.  Steps are timed with CUDA
    events, the checks apart."""
    import numpy as np
    import torch
    from gpucell_gb300 import generator
    from gpucell_gb300.fused import FusedSystem

    cfg = generator.constriction(nx=280, ny=96, nz=72, ncells=100, subdiv=3, layout="random")
    fs = FusedSystem(cfg, noise=args.noise, skin=0.075, compact=True, graph=args.graph)
    S, E = max(1, args.constriction_steps), max(1, args.check_every)
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
    ps_steps, fs_steps = 2, K
    seq_launches = 0
    for c in sub:
        ps = ParticleSystem(c, device=dev, noise=args.noise)
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
        fs.step(2, 1)
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


def cpu_leg(cfg, cpu_steps, parity_steps):
    """The FP64 CPU oracle's leg of the bench (rank 0): `cpu_baseline` times
    `cpu_steps` full oracle steps of the workload on the host cores; `parity`
    steps a small walled channel `parity_steps` times with the oracle as the
    checker beside the fused step.  The oracle is used nowhere else here."""
    from gpucell_gb300.build import build_oracle
    if cpu_steps <= 0 and parity_steps <= 0:
        return None, None
    build_oracle()
    cpu = cpu_baseline(cfg, cpu_steps) if cpu_steps > 0 else None
    par = parity_check(parity_steps) if parity_steps > 0 else None
    return cpu, par


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
            "volume_error": float(abs(g["Vol64"][0] / o.vol[0] - 1)),
            "reference": "FP64 CPU oracle (oracle/oracle.c)"}


def cpu_baseline(cfg, steps):
    """FP64 CPU restatement of the method on all host cores, on `steps` full
    steps of the same workload after one warm-up step."""
    from oracle.binding import Oracle
    threads = os.cpu_count() or 1
    o = Oracle(cfg, noise=True, nthreads=threads)
    o.setup()
    o.step()   # warm-up (page-in, thread start-up)
    t0 = time.perf_counter()
    for _ in range(steps):
        o.step()
    dt = time.perf_counter() - t0
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
    return {"value": cfg.n * steps / dt, "unit": "particle-steps/s", "cores": threads, "kind": "port",
            "sample": f"{steps} full step(s) of the {cfg.n}-particle workload after one warm-up step, FP64, OpenMP",
            "cpu_model": cpu_model(),
            "one_core": {"value": small.n / dt1, "unit": "particle-steps/s",
                         "sample": f"one step of a {small.n}-particle suspension ({small.ncell} cells of "
                                   f"{int(small.npar[0])} vertices), FP64, 1 thread"}}


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
    steps = max(1, min(args.steps, 3))
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
                         "sample": f"{steps} full step(s) of the {cfg.n}-particle workload (capped at 3 of the "
                                   f"{args.steps} requested), FP64, OpenMP"},
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
