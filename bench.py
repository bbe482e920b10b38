#!/usr/bin/env python
"""Throughput of the SDPD + membrane timestep on the 4.2M-particle red-cell
suspension (256x128x128 particles, 200 cells of 2562 vertices, hematocrit
20 %, periodic, thermal noise on).

Prints one JSON line.  `value` is particle-steps/s with the state resident in
HBM; `e2e` is the same metric with the state copied host->device before and
device->host after every step (pinned buffers, the reference's
ParticlesDataReturn set); `roofline` describes the dominant kernel, timed
live with CUDA events; `cpu_baseline` is the FP64 CPU restatement of the
method timed on this machine's cores on a bounded sample.

    python bench.py [--steps K] [--warmup W] [--variant plain]
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
PEAKS_FALLBACK = {"hbm_gbs": 6800.0}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--variant", choices=["plain"], default="plain")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-steps", type=int, default=1)
    ap.add_argument("--small", action="store_true", help="a 1/8-size suspension (for quick checks)")
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


# Dominant kernel: the SDPD pair force.  Algorithmic bytes per particle:
# position 12 + velocity/density 16 + pressure 4 + id 4 + cube 12 read,
# force 12 written.
SDPD_BYTES_PER_PARTICLE = 60


def run_ours(args):
    import numpy as np
    import torch
    import torch.distributed as dist

    from gpucell_gb300 import _lib
    from gpucell_gb300.build import build_library
    from gpucell_gb300.host import ParticleSystem

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

    cfg, wdesc = workload(args, rank)
    ps = ParticleSystem(cfg, device=dev, noise=True)

    def barrier():
        if world > 1:
            dist.barrier()

    for _ in range(max(args.warmup, 3)):
        ps.update()
    torch.cuda.synchronize()

    sampler = ClockSampler()
    if rank == 0:
        sampler.start()
    K = args.steps
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kstart = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    kend = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    barrier()
    torch.cuda.synchronize()
    l0 = _lib.launch_count()
    ev0.record()
    for k in range(K):
        ps.update_coor()
        ps.periodic()
        ps.con_cube_list()
        ps.density()
        ps.predict()
        ps.bound2_vel()
        ps.eos()
        kstart[k].record()
        ps.sdpd_force()
        kend[k].record()
        ps.rep_force()
        ps.ext_force(1)
        ps.cal_geo_para()
        ps.def_force()
        ps.agg_force()
        ps.correct()
        ps.bound2_vel()
        ps.step_count += 1
    ev1.record()
    torch.cuda.synchronize()
    barrier()
    launches = _lib.launch_count() - l0
    t_ms = ev0.elapsed_time(ev1)
    clocks = sampler.stop(local) if rank == 0 else None
    sdpd_ms = sum(a.elapsed_time(b) for a, b in zip(kstart, kend)) / K
    if world > 1:
        t = torch.tensor([t_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_ms = float(t.item())
    flags = _lib.device_status()

    # ---- end to end: host state -> device, one step, results -> host ----
    dyn = ["TotalCoor", "Velrhop", "VelHalf", "TotalForce", "nThroBound", "SortPart"] + \
          (["CurPos"] if ps.has_cells else [])
    outs = ["Press"] + (["Area", "Vol", "DefForce", "AggForce", "TriNorDir", "TriCenter"] if ps.has_cells else [])
    host = {k: torch.empty_like(ps.d[k], device="cpu").pin_memory() for k in dyn + outs}
    for k in dyn:
        host[k].copy_(ps.d[k])
    bi = sum(host[k].numel() * host[k].element_size() for k in dyn)
    bo = sum(host[k].numel() * host[k].element_size() for k in dyn + outs)
    KE = max(1, args.e2e_steps)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for _ in range(KE):
        for k in dyn:
            ps.d[k].copy_(host[k], non_blocking=True)
        ps.update(1)
        for k in dyn + outs:
            host[k].copy_(ps.d[k], non_blocking=True)
        torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    barrier()
    if world > 1:
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())

    n_all = cfg.n * world
    value = n_all * K / (t_ms / 1e3)
    e2e_value = n_all * KE / e2e_s
    peaks, peak_kind = measured_peaks()
    hbm = float(peaks["hbm_gbs"])
    sdpd_bytes = SDPD_BYTES_PER_PARTICLE * cfg.n
    achieved = sdpd_bytes / (sdpd_ms / 1e3) / 1e9
    step_bytes = plain_bytes_per_step(cfg)
    step_gbs = step_bytes / (t_ms / K / 1e3) / 1e9

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return

    cpu = cpu_baseline(cfg, args.cpu_steps) if world == 1 else None
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "particle-steps/s",
        "n_gpus": world,
        "steps": K,
        "warmup": max(args.warmup, 3),
        "ms_per_step": t_ms / K,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32",
        "data": "synthetic (seeded generator, no dataset)",
        "variant": "plain FP32, reference-structured (one kernel per boundary entry point)",
        "config": dict(wdesc, particles=cfg.n, membrane_vertices=cfg.ncp, triangles=cfg.ntri, edges=cfg.nedge,
                       parallelism=f"replicas x{world}" if world > 1 else "single GPU",
                       l2="working set (~0.45 GB of particle state) is larger than L2; no flush",
                       noise="on"),
        "clocks": clocks,
        "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": bi,
                "d2h_bytes_per_step": bo, "steps": KE,
                "path": "reference-facing C ABI (gc_cupar_*/gc_cudiv_*), pinned host buffers"},
        "gpu_launches": launches,
        "roofline": {
            "kernel": "k_sdpd (CalFluidSDPDForce)",
            "bound": "hbm",
            "achieved": achieved,
            "peak": hbm,
            "unit": "GB/s",
            "frac": achieved / hbm,
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback",
            "traffic": None,
            "bytes_per_launch": sdpd_bytes,
            "launch_ms": sdpd_ms,
            "note": "the pair sweep is FP32-issue bound; bytes are 60 per particle",
        },
        "step_roofline": {"bytes_per_step": step_bytes, "achieved_gbs": step_gbs, "frac": step_gbs / hbm,
                          "rule": "352 N + 16 N_tri + 32 N_edge + 28 N_vert"},
        "device_flags": flags,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def cpu_baseline(cfg, steps):
    """FP64 CPU restatement of the method on all host cores, on `steps` full
    steps of the same workload."""
    from oracle.binding import Oracle
    threads = os.cpu_count() or 1
    o = Oracle(cfg, noise=True, nthreads=threads)
    o.setup()
    t0 = time.perf_counter()
    for _ in range(steps):
        o.step()
    dt = time.perf_counter() - t0
    return {"value": cfg.n * steps / dt, "unit": "particle-steps/s", "cores": threads, "kind": "port",
            "sample": f"{steps} full step(s) of the {cfg.n}-particle workload, FP64, OpenMP"}


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
    o.step()   # one warm-up step (page-in, thread start-up)
    steps = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(steps):
        o.step()
    dt = time.perf_counter() - t0
    value = cfg.n * steps / dt
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "particle-steps/s",
        "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": steps,
        "warmup": 1,
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
