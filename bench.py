"""Benchmark: BSSN grid-point RK4 updates/s on GB300 (one JSON line on rank 0).

Workload (N=1): the linearised Teukolsky quadrupole wave on a single 128^3
vertex grid over [-4,4]^3 -- amplitude 1e-5, width 1, 1+log lapse,
Gamma-driver shift (eta=2, g=0.75), KO nu=0.02, Sommerfeld faces, CFL 0.25,
float64 state and arithmetic (the plain FP64 kernels).  A "step" is one RK4
step of the whole grid.  Inputs are synthetic (generated on the host from the
analytic solution).  The resident state is 21 x 136^3 doubles (~420 MB),
larger than the 129 MB L2, so no flush is needed between steps.

Arms:
  --impl gb300 (default)  the CUDA kernels; `value` is device-resident
                          throughput, `e2e` goes through the public rk4_step
                          call with pinned host buffers copied in and out
                          every step.
  --impl reference        the reference algorithm's CPU implementation on the
                          host cores: JAX is not installed, so this is the
                          NumPy restatement of the reference (oracle/), timed
                          on a bounded sample of the same workload.

Multi-GPU (torchrun): independent replicas, one grid per rank (the path has
no exchange step on one box); value = all ranks' updates / max rank time.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "BSSN grid-point RK4 updates/s"
UNIT = "updates/s"
BYTES_PER_UPDATE = 2856          # algorithmic HBM bytes per point per RK4 step (21 comps, 357 doubles)
RHS_AT_BYTES_PER_POINT = 480     # k_rhs_at: 21 state + 33 derivative values read, 6 written (x 8 B)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    return ap.parse_args()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def config_dict(n):
    return {"workload": f"linearised Teukolsky quadrupole wave, {n}^3 vertex grid over [-4,4]^3, FP64 plain kernels",
            "grid": [n, n, n], "amplitude": 1e-5, "width": 1.0, "gauge": "1+log", "shift": "Gamma-driver eta=2 g=0.75",
            "nu": 0.02, "kappa": 0.0, "boundaries": "Sommerfeld on all faces", "cfl": 0.25,
            "l2": "resident state > 129 MB L2; no flush", "parallelism": "replicas"}


# ----------------------------------------------------------------------------
# clocks
# ----------------------------------------------------------------------------

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------
# GB300 arm
# ----------------------------------------------------------------------------

def run_gb300(args, world, rank, local):
    import numpy as np
    import torch

    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=device)

    from jax_bssn_gb300 import _native, build
    if not build.LIBRARY.exists():
        build.build()
    lib = _native.load()
    from jax_bssn_gb300.evolution import PatchEvolution
    from jax_bssn_gb300.evolution.time_evolve import rk4_step
    from jax_bssn_gb300.initial_data import teukolsky_config

    n = args.n
    state, params = teukolsky_config(n=n)
    points = n ** 3

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # ---- device-resident throughput ----
    evo = PatchEvolution(state, params)
    for _ in range(args.warmup):
        evo.step(1)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    launches0 = lib.bssn_launch_count()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(args.steps):
        evo.step(1)
    t1.record(stream)
    torch.cuda.synchronize()
    barrier()
    launches = lib.bssn_launch_count() - launches0
    clock_info = clocks.stop()
    ms = t0.elapsed_time(t1)
    if world > 1:
        t = torch.tensor([ms], device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * points * args.steps / (ms / 1e3)
    nonfinite = evo.nonfinite_count()

    # ---- per-kernel device time (profiled pass, not part of `value`) ----
    lib.bssn_profile_reset()
    lib.bssn_profile_enable(1)
    evo.step(2)
    torch.cuda.synchronize()
    lib.bssn_profile_enable(0)
    prof = _native.profile_read()
    lib.bssn_profile_reset()

    peaks = {}
    peaks_path = ROOT / "MEASURED_PEAKS.json"
    if peaks_path.exists():
        peaks = json.loads(peaks_path.read_text())
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    total_prof = sum(v[0] for v in prof.values()) or 1.0
    dominant = max(prof.items(), key=lambda kv: kv[1][0])
    dom_name, (dom_ms, dom_launches) = dominant
    per_launch_ms = dom_ms / max(dom_launches, 1)
    alg_bytes = points * RHS_AT_BYTES_PER_POINT if dom_name == "rhs_at" else None
    achieved = (alg_bytes / (per_launch_ms / 1e3) / 1e9) if alg_bytes else None
    roofline = {
        "bound": "hbm", "kernel": f"k_{dom_name}", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
        "frac": (achieved / hbm_peak) if achieved else None, "traffic": None,
        "peak_source": peak_src, "kernel_share": dom_ms / total_prof, "kernel_ms_per_launch": per_launch_ms,
        "algorithmic_bytes_per_point": RHS_AT_BYTES_PER_POINT,
        "step_hbm_frac": value / world * BYTES_PER_UPDATE / (hbm_peak * 1e9),
        "note": "plain FP64 form is FP64-pipe bound on GB300; HBM fraction reported as the metric asks",
    }
    kernel_table = {k: {"ms": round(v[0], 3), "launches": v[1], "share": round(v[0] / total_prof, 4)}
                    for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])}

    # ---- end to end through the public API, pinned host buffers ----
    e2e = None
    if not args.no_e2e:
        host = [torch.from_numpy(np.ascontiguousarray(f)).pin_memory() for f in state]
        dev = [h.to(device, non_blocking=True) for h in host]
        h2d = sum(h.numel() * 8 for h in host)
        from jax_bssn_gb300.bssn.variables import BSSNVariables
        torch.cuda.synchronize()
        rk4_step(BSSNVariables(*dev), params)  # warm the workspace cache
        torch.cuda.synchronize()
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            for d, h in zip(dev, host):
                d.copy_(h, non_blocking=True)
            out = rk4_step(BSSNVariables(*dev), params)
            for h, o in zip(host, out):
                h.copy_(o, non_blocking=True)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        ems = e0.elapsed_time(e1)
        if world > 1:
            t = torch.tensor([ems], device=device)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ems = float(t.item())
        e2e = {"value": world * points * args.steps / (ems / 1e3), "unit": UNIT,
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d, "ms_per_step": ems / args.steps}

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(sample_n=36)

    if world > 1:
        torch.distributed.destroy_process_group()
    if rank != 0:
        return None
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (analytic Teukolsky initial data on the host)",
        "config": config_dict(n), "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": launches, "clocks": clock_info, "kernels": kernel_table,
        "nonfinite_after": nonfinite,
    }


# ----------------------------------------------------------------------------
# CPU baseline / reference arm
# ----------------------------------------------------------------------------

def cpu_baseline(sample_n=36, steps=1):
    """The reference algorithm on the host (NumPy restatement, one thread),
    one or more RK4 steps of the same Teukolsky configuration on a smaller grid."""
    from jax_bssn_gb300.initial_data import teukolsky_config
    from oracle import bssn as ob
    from oracle.state import BSSNParameters as OP, BSSNVariables as OV
    state, params = teukolsky_config(n=sample_n)
    s = OV(*state)
    p = OP(**params._asdict())
    t = time.perf_counter()
    for _ in range(steps):
        s = ob.rk4_step(s, p)
    dt = time.perf_counter() - t
    return {"value": sample_n ** 3 * steps / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{steps} RK4 step(s) of the same Teukolsky configuration on a {sample_n}^3 grid "
                      f"(NumPy restatement of the reference, single thread; JAX not installed)",
            "seconds": dt}


def run_reference(args, world, rank):
    if rank != 0:
        return None
    from jax_bssn_gb300.initial_data import teukolsky_config
    from oracle import bssn as ob
    from oracle.state import BSSNParameters as OP, BSSNVariables as OV
    n = 24
    state, params = teukolsky_config(n=n)
    s = OV(*state)
    p = OP(**params._asdict())
    for _ in range(args.warmup):
        s = ob.rk4_step(s, p)
    t = time.perf_counter()
    for _ in range(args.steps):
        s = ob.rk4_step(s, p)
    dt = time.perf_counter() - t
    value = n ** 3 * args.steps / dt
    sample = (f"each step one RK4 step of the Teukolsky configuration on a {n}^3 grid, NumPy restatement "
              "of the reference (the reference's JAX CPU path cannot be installed here), single thread")
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(args.n), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        out = run_reference(args, world, rank)
    else:
        out = run_gb300(args, world, rank, local)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
