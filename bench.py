"""Benchmark: BSSN grid-point RK4 updates/s on GB300 (one JSON line on rank 0).

Default workload (N=1): the linearised Teukolsky quadrupole wave on a single
128^3 vertex grid over [-4,4]^3 -- amplitude 1e-5, width 1, 1+log lapse,
Gamma-driver shift (eta=2, g=0.75), KO nu=0.02, Sommerfeld faces, CFL 0.25,
float64 state and arithmetic (the plain FP64 kernels).  A "step" is one RK4
step of the whole grid.  The resident state is 21 x 136^3 doubles (~420 MB),
larger than the 129 MB L2, so no flush is needed between steps.

Other workloads (--workload):
  fmr           linear wave (A=1e-8, lambda=4) through a 3-level nested 2:1
                hierarchy: root 96^3 periodic on [-8,8)^3, level 1 65^3, level 2
                49^3, stage-synchronous RK4 at dt = 0.25 dx_finest; updates
                count every patch's owned samples.
  axisymmetric  two zero-momentum punctures (Brill-Lindquist, m=0.5 at z=+-1) on
                the compact Cartoon plane 256 x 512, dx=1/32, kappa=0.002, CFL 0.2;
                updates count the 256 x 512 evolved samples.
  puncture      Bowen-York binary initial data: Newton + conjugate gradients on a
                128^3 cell-centred grid (a "step" is one complete solve; the
                metric counts unknowns x Krylov iterations per second).
  puncture_axi  the axisymmetric collision's initial data: Newton + BiCGSTAB on
                the 128 x 256 meridional grid, tolerances 1e-12.
  horizon       apparent-horizon finder on a triaxially stretched Schwarzschild
                slice (M=2, scales 1, 1.25, 1.5, isotropic) stored as a 124^3
                Cartesian volume (dx=0.04): the finder's defaults (12 x 24
                start, refinement to 24 x 48); a "step" is one complete find.
All inputs are synthetic (analytic initial data generated on the host).

Arms:
  --impl gb300 (default)  the CUDA kernels; `value` is device-resident
                          throughput, `e2e` goes through the public step call
                          with pinned host buffers copied in and out every step
                          (one step's downloads overlap the next one's uploads).
  --impl reference        the reference algorithm's CPU implementation on the
                          host cores: JAX is not installed, so this is the
                          NumPy restatement of the reference (oracle/), timed
                          on a bounded sample of the same workload.

Multi-GPU (torchrun): independent replicas, one problem per rank (the path has
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
# Algorithmic HBM bytes per point of one launch, per kernel class (values read + written x 8 B).
CLASS_BYTES = {
    "rhs_curv": 512,       # 21 state + 33 first derivatives read, 10 written (K, Gt, At in one pass)
    "rhs_at": 480,         # 21 state + 33 first derivatives read, 6 written
    "rhs_kgt": 464,        # 21 state + 33 first derivatives read, 4 written
    "rhs_gauge": 328,      # 21 state + 9 first derivatives read, 11 written
    "first_derivs": 352,   # 11 fields read, 33 derivatives written
    "rk4_stage": 714,      # mean of 63, 105, 105, 84 values over the four stages
    # Cartoon class per evolved point: the reconstruction reads 21 compact values and
    # writes the 9-plane support (21 x 9), the collection reads and writes 21 each
    "cartoon": 21 * 8 + 21 * 9 * 8 + 2 * 21 * 8,
}
RHS_CLASSES = ("rhs_curv", "rhs_at", "rhs_kgt", "rhs_gauge", "first_derivs")
# FP32 form: float state and derivatives (4 B), FP64 RHS written (8 B), W and alpha read from the FP64 state
CLASS_BYTES_F32 = {
    "rhs_at": (21 + 33) * 4 + 2 * 8 + 6 * 8,
    "rhs_kgt": (21 + 33) * 4 + 2 * 8 + 4 * 8,
    "rhs_gauge": (21 + 9) * 4 + 2 * 8 + 11 * 8,
    "first_derivs": 11 * 4 + 33 * 4,
}
# Paired FP32 form: the low words of the second-derivative fields it reads
# (At: gt, W, alpha; K/Gt: alpha, beta; first derivatives: all eleven).
CLASS_BYTES_PAIRED_EXTRA = {"rhs_at": 8 * 4, "rhs_kgt": 4 * 4, "first_derivs": 11 * 4}
FLOAT_FORMS = ("fp32", "fp32_paired")
# The compute-roofline kernel of each form and its executed flops per point
# (FMA = 2), from an ncu count of the 96^3 Teukolsky configuration's interior
# launch (DADD + DMUL + 2 DFMA, resp. FADD + FMUL + 2 FFMA over the launch's
# threads): the one-pass K/Gt/At kernel of the FP64 form, the At kernel of the
# FP32 form.
COMPUTE_KERNEL = {"fp64": ("rhs_curv", 2590), "fp32": ("rhs_at", 1890)}
LEAVES = ("conformal_metric", "conformal_factor", "traceless_K", "trace_K", "conformal_connection", "lapse",
          "shift")
# DRAM bytes per evolved point of the dominant kernel class in one RHS
# evaluation (dram__bytes_read.sum + dram__bytes_write.sum over its launches
# divided by the points), from the ncu captures summarised in profiles/
# (workload, form, class) -> (bytes per point, capture).  Traffic grows with
# the points of a launch, so a launch's traffic is this times its points.
MEASURED_TRAFFIC = {
    ("teukolsky", "fp64", "rhs_curv"): (1221, "profiles/traffic_full_size.md (one RK4 step at 128^3)"),
    ("teukolsky", "fp32", "rhs_at"): (410, "profiles/traffic_full_size.md (the FP32 run of the bench at 128^3)"),
    ("fmr", "fp64", "rhs_curv"): (906, "profiles/traffic_full_size.md (one RK4 step, 96^3 + 65^3 + 49^3)"),
    ("fmr", "fp32", "rhs_at"): (534, "profiles/traffic_full_size.md (one RK4 step, 96^3 + 65^3 + 49^3)"),
    ("axisymmetric", "fp64", "cartoon"): (1472, "profiles/traffic_full_size.md (one RK4 step, 256 x 512)"),
    ("axisymmetric", "fp32", "cartoon"): (787, "profiles/traffic_full_size.md (one RK4 step, 256 x 512)"),
}


def nudged(state):
    """The state with every nonzero sample moved one ulp up: the same physics,
    different rounding from the first operation on."""
    import numpy as np
    import torch
    from jax_bssn_gb300.bssn.variables import BSSNVariables
    out = []
    for f in state:
        if isinstance(f, torch.Tensor):
            out.append(torch.where(f != 0, torch.nextafter(f, torch.full_like(f, float("inf"))), f))
        else:
            f = np.asarray(f)
            out.append(np.where(f != 0, np.nextafter(f, np.inf), f))
    return BSSNVariables(*out)


def background(leaf, t):
    """Flat background of a leaf tensor: identity metric, W = alpha = 1, else 0."""
    import torch
    if leaf == "conformal_metric":
        return torch.eye(3, dtype=t.dtype, device=t.device).reshape((3, 3) + (1,) * (t.ndim - 2))
    return 1.0 if leaf in ("conformal_factor", "lapse") else 0.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--workload", choices=("teukolsky", "fmr", "axisymmetric", "puncture", "puncture_axi",
                                           "horizon", "adjoint", "batch"),
                    default="teukolsky")
    ap.add_argument("--n", type=int, default=None, help="grid size (teukolsky n, fmr root n, axisymmetric Nrho)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-graph", action="store_true", help="launch each step's kernels directly (no CUDA graph)")
    ap.add_argument("--no-tune", action="store_true", help="keep the heuristic RHS launch shapes (no autotuning)")
    ap.add_argument("--no-extra", action="store_true",
                    help="default workload only: skip the FMR and axisymmetric measurements on the same line")
    return ap.parse_args()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# ----------------------------------------------------------------------------
# workloads
# ----------------------------------------------------------------------------

class Teukolsky:
    name = "teukolsky"

    def __init__(self, n=None):
        self.n = n or 128

    def config(self):
        n = self.n
        return {"workload": f"linearised Teukolsky quadrupole wave, {n}^3 vertex grid over [-4,4]^3, "
                            "FP64 plain kernels",
                "grid": [n, n, n], "amplitude": 1e-5, "width": 1.0, "gauge": "1+log",
                "shift": "Gamma-driver eta=2 g=0.75", "nu": 0.02, "kappa": 0.0,
                "boundaries": "Sommerfeld on all faces", "cfl": 0.25,
                "l2": "resident state > 129 MB L2; no flush", "parallelism": "replicas"}

    def setup(self, device):
        from jax_bssn_gb300.initial_data import teukolsky_config
        self.state, self.params = teukolsky_config(n=self.n)
        self.points = self.n ** 3

    def resident(self, precision, nudge=False):
        from jax_bssn_gb300.evolution import PatchEvolution
        return PatchEvolution(nudged(self.state) if nudge else self.state, self.params, precision=precision)

    def snapshot(self, evo):
        return [evo.state()]

    def norms(self, evo):
        from jax_bssn_gb300.bssn.constraints import compute_all_constraints, compute_constraint_norms
        return compute_constraint_norms(compute_all_constraints(evo.state(), self.params))

    def host_leaves(self):
        return [f for f in self.state]

    def public_step(self, leaves):
        from jax_bssn_gb300.bssn.variables import BSSNVariables
        from jax_bssn_gb300.evolution.time_evolve import rk4_step
        return list(rk4_step(BSSNVariables(*leaves), self.params))

    def cpu_sample(self, steps=1, n=36):
        from jax_bssn_gb300.initial_data import teukolsky_config
        from oracle import bssn as ob
        from oracle.state import BSSNParameters as OP, BSSNVariables as OV
        state, params = teukolsky_config(n=n)
        s, p = OV(*state), OP(**params._asdict())

        def run(k):
            nonlocal s
            for _ in range(k):
                s = ob.rk4_step(s, p)
        return run, n ** 3, f"RK4 step(s) of the same Teukolsky configuration on a {n}^3 grid"


class NestedFMR:
    name = "fmr"

    def __init__(self, n=None):
        self.root = n or 96

    def config(self):
        from jax_bssn_gb300.fmr import fine_active_shape
        from jax_bssn_gb300.initial_data import fmr_linear_wave_hierarchy
        shapes = [[self.root] * 3] + [list(fine_active_shape(s)) for s in fmr_linear_wave_hierarchy(self.root).patches]
        return {"workload": f"linear wave through a 3-level nested FMR hierarchy, root {self.root}^3 on [-8,8)^3, "
                            "stage-synchronous RK4, FP64 plain kernels",
                "patch_shapes": shapes, "amplitude": 1e-8, "wavelength": 4.0, "gauge": "harmonic, zero shift",
                "mad": True, "cfl": "0.25 of the finest spacing",
                "deviation": "active extents are 2(hi-lo)+1, so 65^3 and 49^3 stand for 64^3 and 48^3",
                "l2": "resident patches (~255 MB) > 129 MB L2; no flush", "parallelism": "replicas"}

    def setup(self, device):
        from jax_bssn_gb300.fmr import initialize_tiled_fmr
        from jax_bssn_gb300.initial_data import fmr_linear_wave_hierarchy, fmr_linear_wave_root, linear_wave_callback
        self.hierarchy = fmr_linear_wave_hierarchy(self.root)
        root = fmr_linear_wave_root(self.root)
        self.states, self.parameters, self.layouts = initialize_tiled_fmr(
            linear_wave_callback(), root, (self.root,) * 3, self.hierarchy)
        self.points = sum(math.prod(l.active_shape) for l in self.layouts)

    def resident(self, precision, nudge=False):
        from jax_bssn_gb300.fmr import FMREvolution
        states = tuple(nudged(s) for s in self.states) if nudge else self.states
        return FMREvolution(states, self.parameters, self.hierarchy, self.layouts, precision=precision)

    def snapshot(self, evo):
        return list(evo.states())

    def norms(self, evo):
        return evo.constraint_norms()

    def host_leaves(self):
        return [leaf.cpu().numpy() for s in self.states for leaf in s]

    def public_step(self, leaves):
        from jax_bssn_gb300.bssn.variables import BSSNVariables
        from jax_bssn_gb300.fmr import fmr_rk4_step
        states = tuple(BSSNVariables(*leaves[7 * p:7 * p + 7]) for p in range(len(self.layouts)))
        out = fmr_rk4_step(states, self.parameters, self.hierarchy, layouts=self.layouts)
        return [leaf for s in out for leaf in s]

    def cpu_sample(self, steps=1, root=24):
        import numpy as np
        from jax_bssn_gb300.initial_data import fmr_linear_wave_hierarchy, fmr_linear_wave_root, linear_wave_state
        from oracle import fmr as of
        from oracle.state import BSSNParameters as OP, BSSNVariables as OV
        h = fmr_linear_wave_hierarchy(root)
        oh = of.FMRHierarchySpec(tuple(of.FMRPatchSpec(s.coarse_lo, s.coarse_hi, parent=s.parent) for s in h.patches),
                                 use_mad=h.use_mad)
        params, shapes = of.patch_parameters(OP(**fmr_linear_wave_root(root)._asdict()), (root,) * 3, oh)
        states = []
        for p, n in zip(params, shapes):
            axes = [o + p.dx * np.arange(m, dtype=np.float64) for o, m in zip((p.x_min, p.y_min, p.z_min), n)]
            X, Y, Z = np.meshgrid(*axes, indexing="ij")
            owned = linear_wave_state(X, Y, Z, 1e-8, 4.0)
            leaves = []
            for leaf in owned:
                full = np.zeros(leaf.shape[:-3] + tuple(m + 2 * of.GUARD for m in n))
                full[(Ellipsis,) + tuple(slice(of.GUARD, of.GUARD + m) for m in n)] = leaf
                leaves.append(full)
            states.append(OV(*leaves))
        states = of.prepare(tuple(states), params, shapes, oh, project=False)

        def run(k):
            nonlocal states
            for _ in range(k):
                states = of.rk4_step(states, params, shapes, oh)
        pts = sum(math.prod(n) for n in shapes)
        return run, pts, f"stage-synchronous RK4 step(s) of the same 3-level hierarchy scaled to a {root}^3 root"


class Axisymmetric:
    name = "axisymmetric"

    def __init__(self, n=None):
        self.nrho = n or 256

    def config(self):
        return {"workload": f"axisymmetric Cartoon head-on punctures (Brill-Lindquist, m=0.5 at z=+-1), compact "
                            f"{self.nrho + 4}x1x{2 * self.nrho}, dx=1/32, FP64 plain kernels",
                "evolved": [self.nrho, 2 * self.nrho], "gauge": "1+log, Gamma-driver eta=2 g=0.75",
                "kappa": 0.002, "nu": 0.02, "cfl": 0.2, "boundaries": "Sommerfeld x-right and z faces",
                "l2": "support state and work (~1.3 GB) > 129 MB L2; no flush", "parallelism": "replicas"}

    def setup(self, device):
        from jax_bssn_gb300.initial_data import brill_lindquist_config
        self.state, self.params = brill_lindquist_config(num_radial_points=self.nrho, r_max=self.nrho / 32.0)
        self.points = self.nrho * 2 * self.nrho

    def resident(self, precision, nudge=False):
        from jax_bssn_gb300.cartoon.axisymmetry import AxisymmetricEvolution
        return AxisymmetricEvolution(nudged(self.state) if nudge else self.state, self.params, precision=precision)

    def snapshot(self, evo):
        return [evo.state()]

    def norms(self, evo):
        from jax_bssn_gb300.cartoon.axisymmetry import compute_axisymmetric_constraint_norms
        return compute_axisymmetric_constraint_norms(evo.constraints(), params=self.params)

    def host_leaves(self):
        return [f for f in self.state]

    def public_step(self, leaves):
        from jax_bssn_gb300.bssn.variables import BSSNVariables
        from jax_bssn_gb300.cartoon.axisymmetry import axisymmetric_rk4_step
        return list(axisymmetric_rk4_step(BSSNVariables(*leaves), self.params))

    def cpu_sample(self, steps=1, nrho=32):
        from jax_bssn_gb300.initial_data import brill_lindquist_config
        from oracle import cartoon as oc
        from oracle.state import BSSNParameters as OP, BSSNVariables as OV
        state, params = brill_lindquist_config(num_radial_points=nrho, r_max=nrho / 8.0)
        s, p = OV(*state), OP(**params._asdict())

        def run(k):
            nonlocal s
            for _ in range(k):
                s = oc.axi_rk4_step(s, p)
        return run, nrho * 2 * nrho, f"RK4 step(s) of the same punctures on a {nrho}x{2 * nrho} compact plane (dx=1/8)"


WORKLOADS = {w.name: w for w in (Teukolsky, NestedFMR, Axisymmetric)}


# ----------------------------------------------------------------------------
# puncture initial data (Newton-Krylov solves)
# ----------------------------------------------------------------------------

PUNCTURE_METRIC = "Bowen-York Newton-Krylov unknown-iterations/s"
PUNCTURE_UNIT = "unknown-iterations/s"
# Algorithmic HBM bytes per unknown of one Krylov iteration, per kernel class.
PUNCTURE_BYTES = {
    False: {"solve_apply": 40,    # CG apply: r, p_prev, dS/du read; p, Ap written
            "solve_update": 48},  # CG update: x, r, p, Ap read; x, r written
    True: {"solve_apply": 96,     # BiCGSTAB p/q (r, rhat, p, q, dS/du read; p, q written) + s/t (r, q, dS/du; s, t)
           "solve_update": 56},   # BiCGSTAB x/r: x, rhat, p, s, t read; x, r written
}


class Puncture:
    """Cartesian Bowen-York binary: 128^3 cell-centred grid on [-12,12]^3 (the
    reference's cell_centered_grid at 128 points), m=0.5 at z=-+1.5 with
    momenta -+0.2 along x, the reference's default tolerances."""
    name = "puncture"
    axisymmetric = False

    def __init__(self, n=None):
        self.n = n or 128
        self.masses = [0.5, 0.5]
        self.positions = [[0.0, 0.0, -1.5], [0.0, 0.0, 1.5]]
        self.momenta = [[0.2, 0.0, 0.0], [-0.2, 0.0, 0.0]]
        self.tol = dict(newton_tolerance=1e-10, max_newton_iterations=12, linear_tolerance=1e-10,
                        max_linear_iterations=1000)

    def config(self):
        return {"workload": f"Bowen-York binary puncture data, Newton + conjugate gradients on a {self.n}^3 "
                            "cell-centred grid over [-12,12]^3, FP64",
                "masses": self.masses, "positions": self.positions, "momenta": self.momenta,
                "tolerances": self.tol, "unknowns": (self.n - 2) ** 3,
                "l2": "each timed solve re-derives its vectors; 10 grid vectors exceed the 129 MB L2 above ~110^3",
                "parallelism": "replicas"}

    def grid(self, device):
        from jax_bssn_gb300.utilities import bowen_york_solver as by
        return by.cell_centered_grid(self.n, 12.0)

    def unknowns(self):
        return (self.n - 2) ** 3

    def cpu_grid(self, n):
        from oracle import puncture as op
        return op.cell_centered_grid(n, 12.0)

    def cpu_solve(self, grid, dx, counts):
        from oracle import puncture as op
        t = self.tol
        return op.solve_conformal_factor(self.masses, self.positions, self.momenta, grid, dx,
                                         t["newton_tolerance"], t["max_newton_iterations"],
                                         t["linear_tolerance"], t["max_linear_iterations"], counts=counts)

    def cpu_unknowns(self, n):
        return (n - 2) ** 3


class PunctureAxi(Puncture):
    """The axisymmetric head-on collision's initial data
    (demos/axisymmetric_blackhole_collision): meridional 128 x 256 grid,
    r_max 12, m=0.5 at z=-+3 with inward momenta 0.05, tolerances 1e-12 and up
    to 100 Newton steps."""
    name = "puncture_axi"
    axisymmetric = True

    def __init__(self, n=None):
        self.n = n or 128
        self.masses = [0.5, 0.5]
        self.positions = [[0.0, 0.0, -3.0], [0.0, 0.0, 3.0]]
        self.momenta = [[0.0, 0.0, 0.05], [0.0, 0.0, -0.05]]
        self.tol = dict(newton_tolerance=1e-12, max_newton_iterations=100, linear_tolerance=1e-12,
                        max_linear_iterations=1000)

    def config(self):
        return {"workload": f"axisymmetric Bowen-York head-on data, Newton + BiCGSTAB on the {self.n} x "
                            f"{2 * self.n} meridional grid, r_max 12, FP64",
                "masses": self.masses, "positions": self.positions, "momenta": self.momenta,
                "tolerances": self.tol, "unknowns": (self.n - 1) * (2 * self.n - 2),
                "l2": "working set (~2.6 MB) stays in L2: the solve is latency bound", "parallelism": "replicas"}

    def grid(self, device):
        from jax_bssn_gb300.utilities import bowen_york_solver as by
        return by.axisymmetric_cell_centered_grid(self.n, 12.0)

    def unknowns(self):
        return (self.n - 1) * (2 * self.n - 2)

    def cpu_grid(self, n):
        from oracle import puncture as op
        return op.axisymmetric_cell_centered_grid(n, 12.0)

    def cpu_solve(self, grid, dx, counts):
        from oracle import puncture as op
        t = self.tol
        return op.solve_axisymmetric_conformal_factor(self.masses, self.positions, self.momenta, grid, dx,
                                                      t["newton_tolerance"], t["max_newton_iterations"],
                                                      t["linear_tolerance"], t["max_linear_iterations"],
                                                      counts=counts)

    def cpu_unknowns(self, n):
        return (n - 1) * (2 * n - 2)


PUNCTURES = {w.name: w for w in (Puncture, PunctureAxi)}
# Executed FP64 flops per unknown of one CG operator launch (DADD + 2 DFMA, from an
# ncu op count of the 128^3 solve: 5.5 DADD, 3.5 DFMA)
CG_APPLY_FLOPS = 12.5
PUNCTURE_CPU_N = {"puncture": 48, "puncture_axi": 64}


def puncture_cpu(wl, solves=1, n=None):
    """The reference algorithm (NumPy restatement with SciPy's Krylov solvers)
    on a smaller grid of the same problem."""
    n = n or PUNCTURE_CPU_N[wl.name]
    grid, dx = wl.cpu_grid(n)
    counts = []
    t = time.perf_counter()
    for _ in range(solves):
        wl.cpu_solve(grid, dx, counts)
    dt = time.perf_counter() - t
    work = wl.cpu_unknowns(n) * sum(counts)
    shape = f"{n}^3" if not wl.axisymmetric else f"{n} x {2 * n}"
    cores = os.cpu_count() or 1
    return {"value": work / dt, "unit": PUNCTURE_UNIT, "cores": cores, "kind": "port",
            "sample": f"{solves} Newton-Krylov solve(s) of the same punctures on the {shape} grid "
                      f"({sum(counts)} Krylov iterations; NumPy restatement with SciPy's Krylov solvers: "
                      f"elementwise work on one thread, dot products through the threaded BLAS on up to {cores} "
                      "cores; JAX not installed)", "seconds": dt}


def run_puncture(args, world, rank, local):
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
    from jax_bssn_gb300.utilities import bowen_york_solver as by
    wl = PUNCTURES[args.workload](args.n)
    grid, dx = wl.grid(device)
    unknowns = wl.unknowns()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def solve(g):
        return by.puncture_solve(wl.masses, wl.positions, wl.momenta, g, dx, axisymmetric=wl.axisymmetric, **wl.tol)

    peaks = {}
    peaks_path = ROOT / "MEASURED_PEAKS.json"
    if peaks_path.exists():
        peaks = json.loads(peaks_path.read_text())
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        r = solve(grid)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    launches0 = lib.bssn_launch_count()
    iterations = 0
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(args.steps):
        r = solve(grid)
        iterations += sum(r.linear_iterations)
    t1.record(stream)
    torch.cuda.synchronize()
    barrier()
    launches = lib.bssn_launch_count() - launches0
    clock_info = clocks.stop()
    ms = _max_over_ranks(t0.elapsed_time(t1), world, device)
    value = world * unknowns * iterations / (ms / 1e3)
    # per-kernel device time of one profiled solve
    lib.bssn_profile_reset()
    lib.bssn_profile_enable(1)
    rp = solve(grid)
    torch.cuda.synchronize()
    lib.bssn_profile_enable(0)
    prof = _native.profile_read()
    lib.bssn_profile_reset()
    its = sum(rp.linear_iterations)
    total = sum(v[0] for v in prof.values()) or 1.0
    kernels = {k: {"ms": round(v[0], 3), "launches": v[1], "share": round(v[0] / total, 4)}
               for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])}
    name = max(PUNCTURE_BYTES[wl.axisymmetric], key=lambda k: prof.get(k, (0.0, 0))[0])
    kms, klaunch = prof.get(name, (0.0, 0))
    per = PUNCTURE_BYTES[wl.axisymmetric][name]
    achieved = per * unknowns * its / (kms / 1e3) / 1e9 if kms > 0 else None
    roofline = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak if achieved else None, "traffic": None, "peak_source": peak_src,
                "kernel_share": kms / total, "kernel_ms_per_launch": kms / max(klaunch, 1),
                "algorithmic_bytes_per_unknown_iteration": per,
                "note": "launches after convergence inside a chunk return at once and are included in the time"}
    compute = None
    if not wl.axisymmetric and kms > 0:
        peak = _native.fma_peak_gflops(_native.PRECISION_F64) / 1e3
        achieved = CG_APPLY_FLOPS * unknowns * its / (kms / 1e3) / 1e12
        compute = {"bound": "fp64", "kernel": "k_cg_apply", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                   "frac": achieved / peak, "flops_per_unknown": CG_APPLY_FLOPS,
                   "peak_source": "measured live by bssn_probe_fma_peak"}
    e2e = None
    if not args.no_e2e:
        host_grid = grid.cpu().pin_memory()
        host_psi = torch.empty(tuple(grid.shape[:-1]), dtype=torch.float64).pin_memory()
        dev_grid = torch.empty_like(grid)
        h2d = host_grid.numel() * 8
        d2h = host_psi.numel() * 8
        torch.cuda.synchronize()
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e_its = 0
        e0.record(stream)
        for _ in range(args.steps):
            dev_grid.copy_(host_grid, non_blocking=True)
            re = solve(dev_grid)
            host_psi.copy_(re.psi, non_blocking=True)
            e_its += sum(re.linear_iterations)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        ems = _max_over_ranks(e0.elapsed_time(e1), world, device)
        e2e = {"value": world * unknowns * e_its / (ems / 1e3), "unit": PUNCTURE_UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": ems / args.steps}
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = puncture_cpu(wl)
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank != 0:
        return None
    return {
        "metric": PUNCTURE_METRIC, "value": value, "unit": PUNCTURE_UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (analytic puncture parameters)",
        "config": {**wl.config(), "step": "one complete Newton-Krylov solve",
                   "newton_steps": len(r.residual_history), "krylov_iterations": r.linear_iterations,
                   "final_residual": r.residual_history[-1]},
        "roofline": roofline, "roofline_compute": compute, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
        "clocks": clock_info, "kernels": kernels,
    }


def run_puncture_reference(args, world, rank):
    if rank != 0:
        return None
    wl = PUNCTURES[args.workload](args.n)
    n = {"puncture": 32, "puncture_axi": 32}[wl.name]
    puncture_cpu(wl, max(args.warmup, 1), n)
    base = puncture_cpu(wl, args.steps, n)
    value = base["value"]
    return {"metric": PUNCTURE_METRIC, "value": value, "unit": PUNCTURE_UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": base["seconds"] * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": wl.config(),
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": PUNCTURE_UNIT, "cores": base["cores"], "kind": "port",
                             "sample": "each step " + base["sample"]},
            "e2e": {"value": value, "unit": PUNCTURE_UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ----------------------------------------------------------------------------
# apparent-horizon finder
# ----------------------------------------------------------------------------

HORIZON_METRIC = "apparent-horizon finds/s"
HORIZON_UNIT = "finds/s"


class Horizon:
    """The reference suite's triaxial case (tests/test_apparent_horizon.py:118-129):
    Schwarzschild M=2 in isotropic slicing pulled back by scales (1, 1.25, 1.5),
    a 124^3 volume with dx=0.04 about the origin, initial radius 0.9 and the
    finder's defaults."""
    name = "horizon"

    def __init__(self, n=None):
        self.dx = 0.04
        self.count = n or 124
        self.scale = (1.0, 1.25, 1.5)
        self.mass = 2.0
        self.initial = 0.9

    def config(self):
        return {"workload": f"apparent-horizon find on a triaxial Schwarzschild slice (M=2, scales 1/1.25/1.5, "
                            f"isotropic) stored as a {self.count}^3 Cartesian volume, dx={self.dx}, FP64",
                "finder": {"n_theta": 12, "n_phi": 24, "max_angular": 48, "tolerance": 1e-8,
                           "initial_radius": self.initial},
                "l2": f"geometry 18 x {self.count}^3 doubles ({18 * 8 * self.count ** 3 / 1e6:.0f} MB) exceeds "
                      "the 129 MB L2", "parallelism": "replicas"}

    def fields(self, count=None):
        import numpy as np
        count = count or self.count
        axis = (np.arange(count) - (count - 1) / 2) * self.dx
        pos = np.meshgrid(axis, axis, axis, indexing="ij")
        st = [f * q for q, f in zip(pos, self.scale)]
        r = np.sqrt(sum(q ** 2 for q in st))
        gamma = np.eye(3).reshape(3, 3, 1, 1, 1) * (1 + self.mass / (2 * r)) ** 4
        f = np.asarray(self.scale)
        gamma = gamma * (f[:, None] * f[None, :]).reshape(3, 3, 1, 1, 1)
        return (axis, axis, axis), np.ascontiguousarray(gamma), np.zeros_like(gamma)


def band_lu_work(n_theta, n_phi):
    """Algorithmic FP64 flops and bytes of one band LU factorisation with the
    right-hand side carried along (the kernel's band widths)."""
    n = n_theta * n_phi
    kl = min(3 * n_phi - 1, n - 1)
    ku2 = min(2 * kl, n - 1)
    flops = 0
    nbytes = 0
    for k in range(n):
        rows = min(n - 1, k + kl) - k          # rows eliminated below the pivot
        cols = min(n - 1, k + ku2) - k + 1     # trailing columns plus the right-hand side
        flops += 2 * rows * cols
        nbytes += 16 * (rows + 1) * cols + 8 * (rows + 1)
    return flops, nbytes


def horizon_cpu(wl, finds=1, count=None):
    """The oracle finder (NumPy; dense Jacobian and LAPACK solve) on the same
    kind of slice."""
    from oracle import horizon as oh
    axes, gamma, kij = wl.fields(count)
    t = time.perf_counter()
    for _ in range(finds):
        res = oh.find_apparent_horizon(axes, gamma, kij, center=(0, 0, 0), initial_radius=wl.initial)
    dt = time.perf_counter() - t
    cores = os.cpu_count() or 1
    return {"value": finds / dt, "unit": HORIZON_UNIT, "cores": cores, "kind": "port",
            "sample": f"{finds} find(s) on the {count or wl.count}^3 volume ({int(res['iterations'])} Newton "
                      f"iterations; NumPy restatement, dense Jacobian and LAPACK solve through the threaded BLAS on "
                      f"up to {cores} cores; JAX not installed)", "seconds": dt, "mass": res["mass"]}


def run_horizon(args, world, rank, local):
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
    from jax_bssn_gb300.utilities import apparent_horizon as ah
    wl = Horizon(args.n)
    axes, gamma_h, kij_h = wl.fields()
    gamma = torch.as_tensor(gamma_h, device=device)
    kij = torch.as_tensor(kij_h, device=device)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def find(g, k):
        return ah.find_apparent_horizon(axes, g, k, center=(0, 0, 0), initial_radius=wl.initial)

    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        res = find(gamma, kij)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    launches0 = lib.bssn_launch_count()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(args.steps):
        res = find(gamma, kij)
    t1.record(stream)
    torch.cuda.synchronize()
    barrier()
    launches = lib.bssn_launch_count() - launches0
    clock_info = clocks.stop()
    ms = _max_over_ranks(t0.elapsed_time(t1), world, device)
    value = world * args.steps / (ms / 1e3)
    # per-kernel-class device time of one profiled find
    lib.bssn_profile_reset()
    lib.bssn_profile_enable(1)
    rp = find(gamma, kij)
    torch.cuda.synchronize()
    lib.bssn_profile_enable(0)
    prof = _native.profile_read()
    lib.bssn_profile_reset()
    total = sum(v[0] for v in prof.values()) or 1.0
    kernels = {k: {"ms": round(v[0], 3), "launches": v[1], "share": round(v[0] / total, 4)}
               for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])}
    # Newton iterations per resolution: one band factorisation each
    flops = nbytes = 0
    for row in rp["convergence"]:
        f, b = band_lu_work(int(row[0]), int(row[1]))
        flops += f * int(row[5])
        nbytes += b * int(row[5])
    sms, slaunch = prof.get("horizon_solve", (0.0, 0))
    hbm_peak, peak_src = 6800.0, "fallback"
    peaks_path = ROOT / "MEASURED_PEAKS.json"
    if peaks_path.exists():
        peaks = json.loads(peaks_path.read_text())
        if "hbm_gbs" in peaks:
            hbm_peak, peak_src = float(peaks["hbm_gbs"]), "measured"
    achieved = nbytes / (sms / 1e3) / 1e9 if sms > 0 else None
    roofline = {"bound": "hbm", "kernel": "k_band_panel", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak if achieved else None, "traffic": None, "peak_source": peak_src,
                "kernel_share": sms / total, "kernel_ms_per_launch": sms / max(slaunch, 1),
                "algorithmic_bytes_per_find": nbytes,
                "note": "band LU in 8-column panels, one dependent launch each (the horizon_solve class also holds "
                        "the back substitution); the band (at most 32 MB) stays in L2, so the factorisation is bound "
                        "by the per-column latency of the panel factorisation, not by HBM or the FP64 pipe"}
    peak = _native.fma_peak_gflops(_native.PRECISION_F64) / 1e3
    fl = flops / (sms / 1e3) / 1e12 if sms > 0 else None
    compute = {"bound": "fp64", "kernel": "k_band_panel", "achieved": fl, "peak": peak, "unit": "TFLOP/s",
               "frac": fl / peak if fl else None, "flops_per_find": flops,
               "peak_source": "measured live by bssn_probe_fma_peak"}
    e2e = None
    if not args.no_e2e:
        torch.cuda.synchronize()
        barrier()
        e0 = time.perf_counter()
        for _ in range(args.steps):
            re = find(gamma_h, kij_h)
        torch.cuda.synchronize()
        ems = (time.perf_counter() - e0) * 1e3
        ems = _max_over_ranks(ems, world, device)
        e2e = {"value": world * args.steps / (ems / 1e3), "unit": HORIZON_UNIT,
               "h2d_bytes_per_step": gamma_h.nbytes + kij_h.nbytes,
               "d2h_bytes_per_step": re["radius"].nbytes + re["expansion"].nbytes, "ms_per_step": ems / args.steps,
               "note": "host NumPy geometry through find_apparent_horizon (pageable copies); host wall clock"}
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = horizon_cpu(wl, 1)
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank != 0:
        return None
    return {
        "metric": HORIZON_METRIC, "value": value, "unit": HORIZON_UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (analytic Schwarzschild slice)",
        "config": {**wl.config(), "step": "one complete find_apparent_horizon call",
                   "mass": res["mass"], "mass_error": abs(res["mass"] / wl.mass - 1),
                   "convergence": [[int(r[0]), int(r[1]), int(r[5])] for r in res["convergence"]],
                   "residual": res["residual"], "audit_residual": res["audit_residual"]},
        "roofline": roofline, "roofline_compute": compute, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
        "clocks": clock_info, "kernels": kernels,
    }


def run_horizon_reference(args, world, rank):
    if rank != 0:
        return None
    wl = Horizon(args.n)
    finds = max(1, min(args.steps, 2))  # about 15 s per find on the host cores
    horizon_cpu(wl, 1)
    base = horizon_cpu(wl, finds)
    value = base["value"]
    return {"metric": HORIZON_METRIC, "value": value, "unit": HORIZON_UNIT, "n_gpus": world, "steps": finds,
            "warmup": 1, "ms_per_step": base["seconds"] * 1e3 / finds, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": wl.config(),
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": HORIZON_UNIT, "cores": base["cores"], "kind": "port",
                             "sample": "each step " + base["sample"]},
            "e2e": {"value": value, "unit": HORIZON_UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


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

def host_round_trips(public_step, dev, host, steps, stream, chunk_bytes=32 << 20):
    """`steps` calls of a public step, each fed from and returned to pinned host
    memory: the first step's inputs are copied in, every step's outputs are
    copied out to `host`, and those host copies are the next step's inputs.
    Each output chunk goes back in as soon as it has reached the host, on a
    second copy stream, so the downloads of one step and the uploads of the
    next overlap (the two directions share the host link at about 169 GB/s
    each against 192-210 GB/s alone).  Every step still moves all of its
    inputs and outputs through host memory."""
    import torch
    d2h, h2d = torch.cuda.Stream(), torch.cuda.Stream()
    for d, h in zip(dev, host):
        d.copy_(h, non_blocking=True)
    for i in range(steps):
        if i:
            stream.wait_stream(h2d)
        out = public_step(dev)
        done = torch.cuda.Event()
        done.record(stream)
        d2h.wait_event(done)
        last = i == steps - 1
        for o, h, d in zip(out, host, dev):
            if not o.is_contiguous() or o.numel() != h.numel():
                raise RuntimeError("public step outputs must be contiguous and shaped like its inputs")
            o.record_stream(d2h)
            of, hf, df = o.view(-1), h.view(-1), d.view(-1)
            step = max(1, chunk_bytes // o.element_size())
            for a in range(0, of.numel(), step):
                with torch.cuda.stream(d2h):
                    hf[a:a + step].copy_(of[a:a + step], non_blocking=True)
                if not last:
                    arrived = torch.cuda.Event()
                    arrived.record(d2h)
                    h2d.wait_event(arrived)
                    with torch.cuda.stream(h2d):
                        df[a:a + step].copy_(hf[a:a + step], non_blocking=True)
    stream.wait_stream(d2h)


def _max_over_ranks(ms, world, device):
    if world == 1:
        return ms
    import torch
    t = torch.tensor([ms], device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def compute_roofline_of(prof, points, profiled_steps, peak_gflops, precision):
    """FP64 / FP32 pipe roofline of the form's curvature kernel: executed flops
    of its launches in the profiled steps over their summed device time, against
    the live FMA peak (forms without a flop count give none)."""
    if precision not in COMPUTE_KERNEL:
        return None
    name, per_point = COMPUTE_KERNEL[precision]
    if name not in prof or not peak_gflops:
        return None
    ms, launches = prof[name]
    flops = per_point * points * 4 * profiled_steps
    achieved = flops / (ms / 1e3) / 1e12
    peak = peak_gflops / 1e3
    return {"bound": precision, "kernel": f"k_{name}", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "flops_per_point": per_point,
            "peak_source": "measured live by bssn_probe_fma_peak"}


def roofline_of(prof, points, profiled_steps, hbm_peak, peak_src, value_per_gpu, precision="fp64", workload=None):
    """Live roofline of the dominant kernel class from the per-launch CUDA-event
    accounting: algorithmic bytes of all its launches in the profiled steps
    divided by their summed device time."""
    total = sum(v[0] for v in prof.values()) or 1.0
    name, (ms, launches) = max(prof.items(), key=lambda kv: kv[1][0])
    per_point = CLASS_BYTES.get(name)
    if per_point is not None and precision in FLOAT_FORMS and name in RHS_CLASSES:
        per_point = CLASS_BYTES_F32.get(name)
        if per_point is not None and precision == "fp32_paired":
            per_point += CLASS_BYTES_PAIRED_EXTRA.get(name, 0)
    achieved = None
    if per_point is not None and ms > 0:
        alg = per_point * points * 4 * profiled_steps
        achieved = alg / (ms / 1e3) / 1e9
    measured = MEASURED_TRAFFIC.get((workload, precision, name))
    traffic = {}
    if measured:
        traffic = {"traffic_bytes_per_point": measured[0], "traffic_source": measured[1],
                   "traffic_over_algorithmic": measured[0] / per_point if per_point else None}
    return {
        "bound": "hbm", "kernel": f"k_{name}", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
        "frac": (achieved / hbm_peak) if achieved else None,
        "traffic": measured[0] * points if measured else None, **traffic, "peak_source": peak_src,
        "kernel_share": ms / total, "kernel_ms_per_launch": ms / max(launches, 1),
        "algorithmic_bytes_per_point": per_point,
        "step_hbm_frac": value_per_gpu * BYTES_PER_UPDATE / (hbm_peak * 1e9),
        "note": ("plain FP64 form is FP64-pipe bound on GB300; HBM fraction reported as the metric asks"
                 if precision == "fp64" else "FP32-arithmetic form: float reads of the state and derivatives"),
    }


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

    wl = WORKLOADS[args.workload](args.n)
    wl.setup(device)
    points = wl.points

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    peaks = {}
    peaks_path = ROOT / "MEASURED_PEAKS.json"
    if peaks_path.exists():
        peaks = json.loads(peaks_path.read_text())
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    stream = torch.cuda.current_stream()
    fma_peaks = {"fp64": _native.fma_peak_gflops(_native.PRECISION_F64),
                 "fp32": _native.fma_peak_gflops(_native.PRECISION_F32)}

    def measure(wl, precision, steps):
        """Device-resident throughput of one arithmetic form, its per-kernel
        profile and live roofline, and end-to-end public-API throughput."""
        points = wl.points
        evo = wl.resident(precision)
        launch_shapes = None
        if not args.no_tune and hasattr(evo, "tune"):
            launch_shapes = evo.tune()      # autotuned RHS block sizes (untimed)
        for _ in range(args.warmup):
            evo.step(1)
        if not args.no_graph:
            # one RK4 step as a CUDA graph, replayed once per timed step
            evo.capture(1)
            evo.step(1)
        torch.cuda.synchronize()
        clocks = ClockSampler(local)
        clocks.start()
        barrier()
        torch.cuda.synchronize()
        launches0 = lib.bssn_launch_count()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(steps):
            evo.step(1)
        t1.record(stream)
        torch.cuda.synchronize()
        barrier()
        launches = lib.bssn_launch_count() - launches0
        if evo.captured:
            # replays bypass the host-side counter: each runs the captured launches
            launches += evo.graph_launches * steps
            evo.release_graph()
        clock_info = clocks.stop()
        ms = _max_over_ranks(t0.elapsed_time(t1), world, device)
        value = world * points * steps / (ms / 1e3)
        # per-kernel device time (profiled pass, not part of `value`)
        profiled_steps = 2
        lib.bssn_profile_reset()
        lib.bssn_profile_enable(1)
        evo.step(profiled_steps)
        torch.cuda.synchronize()
        lib.bssn_profile_enable(0)
        prof = _native.profile_read()
        lib.bssn_profile_reset()
        roofline = roofline_of(prof, points, profiled_steps, hbm_peak, peak_src, value / world, precision, wl.name)
        compute = compute_roofline_of(prof, points, profiled_steps, fma_peaks.get(precision), precision)
        total_prof = sum(v[0] for v in prof.values()) or 1.0
        kernels = {k: {"ms": round(v[0], 3), "launches": v[1], "share": round(v[0] / total_prof, 4)}
                   for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])}
        e2e = None
        if not args.no_e2e:
            import jax_bssn_gb300 as pkg
            host = [torch.from_numpy(np.ascontiguousarray(f)).pin_memory() for f in wl.host_leaves()]
            dev = [h.to(device, non_blocking=True) for h in host]
            h2d = sum(h.numel() * h.element_size() for h in host)
            with pkg.arithmetic(precision):
                torch.cuda.synchronize()
                wl.public_step(dev)  # warm the workspace cache
                torch.cuda.synchronize()
                barrier()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                host_round_trips(wl.public_step, dev, host, steps, stream)
                e1.record(stream)
                torch.cuda.synchronize()
                barrier()
            ems = _max_over_ranks(e0.elapsed_time(e1), world, device)
            e2e = {"value": world * points * steps / (ems / 1e3), "unit": UNIT,
                   "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d, "ms_per_step": ems / steps}
        steps_total = args.warmup + (0 if args.no_graph else 1) + steps + profiled_steps
        return {"evo": evo, "value": value, "ms": ms, "launches": launches, "clocks": clock_info,
                "roofline": roofline, "compute": compute, "kernels": kernels, "e2e": e2e,
                "launch_shapes": launch_shapes or "heuristic (set_threads)", "steps_total": steps_total,
                "precision": precision}

    def both_forms(wl, steps):
        """The FP64 run, both float forms, and the FP64 run-to-run spread of the
        constraint norms (a second FP64 run from the initial data nudged one ulp,
        advanced the same number of steps, untimed)."""
        plain = measure(wl, "fp64", steps)
        floats = {form: measure(wl, form, steps) for form in FLOAT_FORMS}
        twin = wl.resident("fp64", nudge=True)
        twin.step(plain["steps_total"])
        torch.cuda.synchronize()
        comparison = compare_forms(wl, plain, floats, wl.norms(twin), steps)
        del twin
        chosen = floats[comparison["form"]]
        return plain, floats, chosen, comparison

    plain, floats, chosen, chosen_form = both_forms(wl, args.steps)
    value, ms, launches, clock_info = plain["value"], plain["ms"], plain["launches"], plain["clocks"]
    roofline, kernel_table, e2e = plain["roofline"], plain["kernels"], plain["e2e"]

    # The nested-FMR and axisymmetric workloads ride along on the default line
    # (each a few seconds), so every evolution configuration is measured by
    # the same run.
    extra = {}
    if args.workload == "teukolsky" and args.n is None and not args.no_extra:
        for name in ("fmr", "axisymmetric"):
            other = WORKLOADS[name](None)
            other.setup(device)
            p64, pf, _, form = both_forms(other, args.steps)
            extra[name] = {"config": other.config(), "value": p64["value"], "unit": UNIT,
                           "ms_per_step": p64["ms"] / args.steps, "roofline": p64["roofline"],
                           "roofline_compute": p64["compute"], "e2e": p64["e2e"], "gpu_launches": p64["launches"],
                           "clocks": p64["clocks"], "kernels": p64["kernels"], "chosen_form": form}
            del p64, pf, other
            torch.cuda.empty_cache()
        if world == 1:
            # the other workloads, shortened, so the driver's run measures them too
            # (each carries its own config, timing and launches; none is part of
            # the headline's timed region)
            for name, runner, over in (
                    ("adjoint", run_adjoint, dict(steps=1, warmup=1, adjoint_steps=20, adjoint_fd=1, no_e2e=True)),
                    ("batch", run_batch, dict(steps=5, warmup=2)),
                    ("puncture", run_puncture, dict(steps=3, warmup=1)),
                    ("horizon", run_horizon, dict(steps=5, warmup=2))):
                sub = argparse.Namespace(**vars(args))
                sub.workload, sub.n, sub.no_cpu = name, None, True
                for key, val in over.items():
                    setattr(sub, key, val)
                out = runner(sub, world, rank, local)
                extra[name] = {k: out[k] for k in (
                    "metric", "value", "unit", "steps", "ms_per_step", "config", "roofline", "roofline_compute",
                    "e2e", "gpu_launches", "clocks", "kernels", "forward_ms", "backward_ms", "adjoint_over_forward",
                    "gradient_over_forward", "fd_check", "by_grid_and_batch") if k in out}
                torch.cuda.empty_cache()

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(wl)

    if world > 1:
        torch.distributed.destroy_process_group()
    if rank != 0:
        return None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (analytic initial data generated on the host)",
        "config": {**wl.config(), "execution": ("direct kernel launches" if args.no_graph else
                                                "each timed step replays one RK4 step captured as a CUDA graph")},
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": launches, "clocks": clock_info, "kernels": kernel_table,
        "roofline_compute": plain["compute"], "fma_peaks_gflops": fma_peaks, "chosen_form": chosen_form,
        "launch_shapes": {"fp64": plain["launch_shapes"], **{f: m["launch_shapes"] for f, m in floats.items()}},
    }
    if extra:
        line["workloads"] = extra
    return line


FORM_ARITHMETIC = {
    "fp32": "FP32 RHS stencils and algebra on perturbations about the flat background; FP64 state, RK4 "
            "combination, projection, W/alpha/1/W and constraints",
    "fp32_paired": "as fp32, with gt, W, alpha and beta held as float pairs hi + lo for their derivatives "
                   "(their 1/dx^2-amplified rounding at about FP64's)",
}


def compare_forms(wl, plain, floats, twin_norms, steps):
    """Each float form against the FP64 run after the same number of steps, and
    the choice: the fastest form whose Hamiltonian and momentum L2 norms are
    within max(1%, twice the FP64 run-to-run spread) of the FP64 run's."""
    import torch
    n64 = wl.norms(plain["evo"])
    norm_keys = [k for k in ("hamiltonian_l2", "momentum_l2") if k in n64]
    rel = lambda a, b: abs(a - b) / abs(b) if b else None
    spread = {k: rel(twin_norms[k], n64[k]) for k in norm_keys}
    bar = {k: max(0.01, 2.0 * (spread[k] or 0.0)) for k in norm_keys}
    forms = {}
    for form, m in floats.items():
        # error against the FP64 run relative to each leaf's deviation from the
        # flat background (signal = that deviation's maximum, abs = the maximum
        # difference; a leaf whose signal is itself at roundoff level, such as K
        # and the connection functions of a transverse-traceless wave, has a
        # ratio near one by nature)
        errors = {}
        for s64, s32 in zip(wl.snapshot(plain["evo"]), wl.snapshot(m["evo"])):
            for leaf, a, b in zip(LEAVES, s64, s32):
                dev64 = a - background(leaf, a)
                scale = float(torch.max(torch.abs(dev64)))
                err = float(torch.max(torch.abs(b - a)))
                e = errors.setdefault(leaf, {"rel": 0.0, "abs": 0.0, "signal": 0.0})
                e["rel"] = max(e["rel"], err / scale if scale > 0 else err)
                e["abs"], e["signal"] = max(e["abs"], err), max(e["signal"], scale)
        nf = wl.norms(m["evo"])
        norms = {k: {"fp64": n64[k], form: nf[k], "rel_diff": rel(nf[k], n64[k])} for k in norm_keys}
        meets = all(norms[k]["rel_diff"] is not None and norms[k]["rel_diff"] <= bar[k] for k in norm_keys)
        forms[form] = {
            "arithmetic": FORM_ARITHMETIC[form], "dtype": "f32 (f64 state)", "value": m["value"], "unit": UNIT,
            "ms_per_step": m["ms"] / steps, "speedup_vs_fp64": m["value"] / plain["value"],
            "roofline": m["roofline"], "roofline_compute": m["compute"], "e2e": m["e2e"],
            "gpu_launches": m["launches"], "clocks": m["clocks"], "kernels": m["kernels"],
            "error_vs_fp64": {"metric": "per leaf rel = abs / signal, abs = max|form - fp64|, signal = "
                                        f"max|fp64 - background|, after {m['steps_total']} steps",
                              "per_leaf": errors},
            "constraint_norms": norms, "meets_bar": meets,
        }
    passing = [f for f in forms if forms[f]["meets_bar"]]
    form = max(passing or forms, key=lambda f: forms[f]["value"])
    return {
        "form": form, **forms[form],
        "choice": ("fastest float form within the bar" if passing else
                   "no float form within the bar: the fastest is reported, FP64 stays the headline"),
        "bar": {"rule": "rel_diff <= max(0.01, 2 x fp64_spread) for each norm", **bar},
        "fp64_spread": {"metric": "rel. difference of the FP64 run's norms and those of a second FP64 run from "
                                  "the initial data with every nonzero sample one ulp up, same steps",
                        **spread},
        "forms": {f: {k: v for k, v in forms[f].items()
                      if k in ("value", "ms_per_step", "speedup_vs_fp64", "constraint_norms", "meets_bar", "e2e")}
                  for f in forms},
    }
# ----------------------------------------------------------------------------
# CPU baseline / reference arm
# ----------------------------------------------------------------------------

# The reference's CPU path is the NumPy restatement (JAX cannot be installed
# here; the restatement reproduces the reference source's goldens bit for
# bit).  NumPy runs one thread per process, so the host's cores run one
# independent instance of a smaller grid of the same configuration each, in
# processes started with `spawn` (no CUDA state is inherited).
_POOL_STATE = {}


def _pool_init(workload, kwargs):
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    sys.path.insert(0, str(ROOT))
    wl = WORKLOADS[workload](None)
    run, pts, what = wl.cpu_sample(**kwargs)
    _POOL_STATE.update(run=run, pts=pts, what=what)


def _pool_step(steps):
    t = time.perf_counter()
    _POOL_STATE["run"](steps)
    return time.perf_counter() - t, _POOL_STATE["pts"], _POOL_STATE["what"]


CPU_SAMPLE = {"teukolsky": {"n": 40}, "fmr": {"root": 24}, "axisymmetric": {"nrho": 32}}


class HostInstances:
    """One oracle instance per host core; `step(k)` advances all of them k
    RK4 steps at once and returns (wall seconds, points per instance, what)."""

    def __init__(self, workload, cores=None):
        import multiprocessing as mp
        self.cores = cores or os.cpu_count() or 1
        env_threads = {k: os.environ.get(k) for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")}
        for k in env_threads:
            os.environ[k] = "1"
        ctx = mp.get_context("spawn")
        self.pool = ctx.Pool(self.cores, initializer=_pool_init, initargs=(workload, CPU_SAMPLE[workload]))
        for k, v in env_threads.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v

    def step(self, steps=1):
        t = time.perf_counter()
        out = self.pool.map(_pool_step, [steps] * self.cores, chunksize=1)
        return time.perf_counter() - t, out[0][1], out[0][2]

    def close(self):
        self.pool.close()
        self.pool.join()


def sample_config(wl, cores, what):
    """The configuration that ran on the host: the workload's own keys, with
    the sample's grid in place of the benchmarked one."""
    cfg = dict(wl.config())
    small = CPU_SAMPLE[wl.name]
    if wl.name == "teukolsky":
        cfg["grid"] = [small["n"]] * 3
    elif wl.name == "fmr":
        from jax_bssn_gb300.fmr import fine_active_shape
        from jax_bssn_gb300.initial_data import fmr_linear_wave_hierarchy
        root = small["root"]
        cfg["patch_shapes"] = [[root] * 3] + [list(fine_active_shape(s))
                                              for s in fmr_linear_wave_hierarchy(root).patches]
    elif wl.name == "axisymmetric":
        cfg["evolved"] = [small["nrho"], 2 * small["nrho"]]
    cfg["workload"] = (f"host sample of the benchmarked configuration: {cores} concurrent instances, one per core, "
                       f"each {what}")
    cfg["instances"] = cores
    cfg["sample_of"] = wl.config()["workload"]
    return cfg


def cpu_baseline(wl, steps=1):
    """The reference algorithm (NumPy restatement) on every host core, one
    instance of a smaller grid of the same configuration per core: one warm-up
    and one timed RK4 step."""
    host = HostInstances(wl.name)
    try:
        host.step(1)
        dt, pts, what = host.step(steps)
    finally:
        host.close()
    return {"value": host.cores * pts * steps / dt, "unit": UNIT, "cores": host.cores, "kind": "port",
            "sample": f"{steps} RK4 step(s) of {host.cores} concurrent instances, one per core, each {what} "
                      "(NumPy restatement of the reference; JAX not installed)",
            "seconds": dt}


def run_reference(args, world, rank):
    if rank != 0:
        return None
    wl = WORKLOADS[args.workload](args.n)
    host = HostInstances(wl.name)
    try:
        for _ in range(args.warmup):
            host.step(1)
        dt = 0.0
        for _ in range(args.steps):
            step_dt, pts, what = host.step(1)
            dt += step_dt
    finally:
        host.close()
    value = host.cores * pts * args.steps / dt
    sample = (f"each step one RK4 step of {host.cores} concurrent instances, one per host core, each {what}; "
              "NumPy restatement of the reference (its JAX CPU path cannot be installed here)")
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": sample_config(wl, host.cores, what), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": host.cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ----------------------------------------------------------------------------
# adjoint (reverse-mode gradient) and instance batches
# ----------------------------------------------------------------------------

ADJOINT_METRIC = "BSSN reverse-mode gradient, grid-point RK4 steps/s (forward + adjoint)"
# Executed FP64 flops per point of one k_adj_point launch (DFMA x 2 + DMUL + DADD,
# ncu on the 32^3 x 4 gauge-wave case, profiles/k_adj_point_gauge_wave.md) and its
# algorithmic bytes (21 state + 33 inner derivatives + 21 RHS adjoint read;
# 21 state adjoint + 111 coefficients written).
ADJ_POINT_FLOPS = 4762
ADJ_POINT_BYTES = 8 * (21 + 33 + 21 + 21 + 111)


def _gauge_wave_batch(n, seeds, device):
    """C5 inputs: the periodic gauge wave with a seeded symmetric 1e-3 Gaussian
    perturbation of gt_ij per seed (numpy default_rng(seed)), component form."""
    import numpy as np
    import torch
    from jax_bssn_gb300.evolution.adjoint import components
    from jax_bssn_gb300.initial_data import gauge_wave_config
    state, params = gauge_wave_config(n=n)
    base = components(state).to(device)
    batch = []
    for seed in range(seeds):
        rng = np.random.default_rng(seed)
        u = base.clone()
        u[0:6] += torch.as_tensor(1e-3 * rng.standard_normal((6, n, n, n)), device=device)
        batch.append(u)
    return torch.stack(batch, dim=1).contiguous(), base, params


def run_adjoint(args, world, rank, local):
    import torch
    from jax_bssn_gb300 import _native
    from jax_bssn_gb300.evolution import BatchEvolution
    from jax_bssn_gb300.evolution.adjoint import CheckpointedEvolution, leaves
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    lib = _native.load()
    # evolution length and finite-difference directions: configuration 5 by
    # default; the default bench line runs a shorter evolution of the same batch
    n, seeds, nsteps = args.n or 64, 16, getattr(args, "adjoint_steps", 200)
    fd_directions = getattr(args, "adjoint_fd", 2)
    u0, base, params = _gauge_wave_batch(n, seeds, device)
    points = seeds * n ** 3
    stream = torch.cuda.current_stream()

    def ev():
        return torch.cuda.Event(enable_timing=True)

    # the plain forward: the same batch, one captured RK4 step replayed
    plain = BatchEvolution([leaves(u0[:, i]) for i in range(seeds)], params)
    plain.step(1)
    plain.capture(1)
    plain.step(1)
    target = BatchEvolution([leaves(base)], params)
    target.step(nsteps)
    from jax_bssn_gb300.evolution.adjoint import components
    w_target = components(target.state(0))[6]
    del target

    def loss_adjoint(final):
        ybar = torch.zeros_like(final)
        ybar[6] = final[6] - w_target
        return ybar

    for _ in range(args.warmup):          # short gradients warm every kernel
        run = CheckpointedEvolution(u0, params, 4, store_stages=2)
        run.backward(loss_adjoint(run.forward()))
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    t = [ev() for _ in range(3)]
    t[0].record(stream)
    plain.step(nsteps)
    t[1].record(stream)
    torch.cuda.synchronize()
    plain_ms = t[0].elapsed_time(t[1])
    fwd_ms = bwd_ms = 0.0
    launches0 = lib.bssn_launch_count()
    run = None
    for _ in range(args.steps):
        run = None                        # one workspace at a time (~170 GB at 64^3 x 16)
        run = CheckpointedEvolution(u0, params, nsteps, store_stages=2)
        t[0].record(stream)
        final = run.forward()
        t[1].record(stream)
        grad = run.backward(loss_adjoint(final))
        t[2].record(stream)
        torch.cuda.synchronize()
        fwd_ms += t[0].elapsed_time(t[1])
        bwd_ms += t[1].elapsed_time(t[2])
    launches = lib.bssn_launch_count() - launches0
    clock_info = clocks.stop()
    memory_gb = run.ws.numel() / 1e9
    run = final = None
    torch.cuda.empty_cache()
    value = points * nsteps * args.steps / ((fwd_ms + bwd_ms) / 1e3)
    # roofline of the dominant adjoint kernel, from a profiled VJP pass
    from jax_bssn_gb300.evolution.adjoint import rhs_vjp
    lib.bssn_profile_reset()
    lib.bssn_profile_enable(1)
    rhs_vjp(u0, torch.randn_like(u0), params)
    torch.cuda.synchronize()
    lib.bssn_profile_enable(0)
    prof = _native.profile_read()
    lib.bssn_profile_reset()
    point_ms = prof.get("adjoint_point", (0.0, 1))[0]
    fma = _native.fma_peak_gflops(_native.PRECISION_F64)
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    roofline = {"bound": "hbm", "kernel": "k_adj_point", "achieved": ADJ_POINT_BYTES * points / (point_ms / 1e3) / 1e9,
                "peak": hbm_peak, "unit": "GB/s", "frac": ADJ_POINT_BYTES * points / (point_ms / 1e3) / 1e9 / hbm_peak,
                "traffic": None, "algorithmic_bytes_per_point": ADJ_POINT_BYTES,
                "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
                "note": "FP64-pipe bound; see roofline_compute"}
    roofline_compute = {"bound": "fp64", "kernel": "k_adj_point",
                        "achieved": ADJ_POINT_FLOPS * points / (point_ms / 1e3) / 1e12, "peak": fma / 1e3,
                        "unit": "TFLOP/s", "frac": ADJ_POINT_FLOPS * points / (point_ms / 1e3) / 1e12 / (fma / 1e3),
                        "flops_per_point": ADJ_POINT_FLOPS, "peak_source": "measured live by bssn_probe_fma_peak"}
    # gradient check: central differences (h = 1e-6) along smooth directions
    # of the metric perturbation, on the full configuration
    import numpy as np

    def loss_of(u):
        run_ = BatchEvolution([leaves(u[:, i]) for i in range(seeds)], params)
        run_.step(nsteps)
        final_ = torch.stack([components(run_.state(i)) for i in range(seeds)], dim=1)
        return 0.5 * float(((final_[6] - w_target) ** 2).sum())

    axes = [torch.arange(n, device=device, dtype=torch.float64) * (2 * np.pi / n)] * 3
    X, Y, Z = torch.meshgrid(*axes, indexing="ij")
    checks = []
    for k in range(fd_directions):
        d = torch.zeros_like(u0)
        for c in range(6):
            d[c] = torch.sin(X + 0.7 * c + k) + 0.5 * torch.cos(2 * Y - c) + 0.3 * torch.sin(Z + X + 1.3 * k)
        h = 1e-6
        fd = (loss_of(u0 + h * d) - loss_of(u0 - h * d)) / (2 * h)
        ad = float((grad * d).sum())
        checks.append({"adjoint": ad, "central_difference": fd, "rel_diff": abs(ad - fd) / abs(fd)})
    # end to end: the initial batch from pinned host memory, the gradient back
    e2e = None
    if not args.no_e2e:
        host_u = u0.cpu().pin_memory()
        host_g = torch.empty_like(host_u).pin_memory()
        e0, e1 = ev(), ev()
        e0.record(stream)
        dev_u = host_u.to(device, non_blocking=True)
        run = CheckpointedEvolution(dev_u, params, nsteps, store_stages=2)
        g = run.backward(loss_adjoint(run.forward()))
        run = None
        host_g.copy_(g, non_blocking=True)
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_ms = e0.elapsed_time(e1)
        nbytes = host_u.numel() * 8
        e2e = {"value": points * nsteps / (e2e_ms / 1e3), "unit": "point-steps/s", "h2d_bytes_per_step": nbytes,
               "d2h_bytes_per_step": nbytes, "ms_per_step": e2e_ms}
    return {
        "metric": ADJOINT_METRIC, "value": value, "unit": "point-steps/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": (fwd_ms + bwd_ms) / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded perturbations)",
        "config": {"workload": f"adjoint of the {n}^3 periodic gauge wave (A=0.1, nu=0.1, CFL 0.25), "
                               f"{seeds} seeds in one batch, {nsteps} RK4 steps; loss 1/2 |W_N - W_target|^2 "
                               "with W_target from the unperturbed run; gradient w.r.t. the seeded 1e-3 Gaussian "
                               "perturbation of gt_ij",
                   "grid": [n, n, n], "instances": seeds, "evolution_steps": nsteps,
                   "checkpointing": f"sqrt(N): segments of ceil(sqrt({nsteps})) steps, stage RHS values and "
                                    "stage states kept while a segment is re-run",
                   "workspace_gb": memory_gb, "step": "one complete gradient (forward + backward)",
                   "l2": "working set > 129 MB L2; no flush"},
        "forward_ms": plain_ms, "recorded_forward_ms": fwd_ms / args.steps, "backward_ms": bwd_ms / args.steps,
        "adjoint_over_forward": (bwd_ms / args.steps) / plain_ms,
        "gradient_over_forward": ((fwd_ms + bwd_ms) / args.steps) / plain_ms,
        "fd_check": checks, "roofline": roofline, "roofline_compute": roofline_compute,
        "kernels_rhs_vjp": {k: {"ms": round(v[0], 3), "launches": v[1]} for k, v in prof.items()},
        "e2e": e2e, "gpu_launches": launches, "clocks": clock_info, "cpu_baseline": None,
    }


def run_batch(args, world, rank, local):
    """Updates/s against batch size: the periodic gauge wave (64^3 and 32^3),
    each timed step one captured RK4 step of the whole batch."""
    import torch
    from jax_bssn_gb300 import _native
    from jax_bssn_gb300.evolution import BatchEvolution
    from jax_bssn_gb300.initial_data import gauge_wave_config
    torch.cuda.set_device(local)
    lib = _native.load()
    stream = torch.cuda.current_stream()
    table, headline = {}, None
    clocks = ClockSampler(local)
    clocks.start()
    launches = 0
    for n in (32, 64):
        state, params = gauge_wave_config(n=n)
        table[n] = {}
        for b in (1, 2, 4, 8, 16):
            evo = BatchEvolution([state] * b, params)
            if not args.no_tune:
                evo.tune()
            for _ in range(args.warmup):
                evo.step(1)
            evo.capture(1)
            evo.step(1)
            torch.cuda.synchronize()
            t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0.record(stream)
            evo.step(args.steps)
            t1.record(stream)
            torch.cuda.synchronize()
            ms = t0.elapsed_time(t1)
            launches += evo.graph_launches * args.steps
            table[n][b] = {"updates_per_s": b * n ** 3 * args.steps / (ms / 1e3), "ms_per_step": ms / args.steps,
                           "launches_per_step": evo.graph_launches}
            del evo
            torch.cuda.empty_cache()
    headline = table[64][16]
    return {"metric": METRIC, "value": headline["updates_per_s"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": headline["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "instance batches of the periodic gauge wave (A=0.1, harmonic, zero shift, "
                                   "nu=0.1, CFL 0.25); value at 64^3 x 16 instances",
                       "grids": [32, 64], "batches": [1, 2, 4, 8, 16],
                       "execution": "each timed step replays one captured RK4 step of the whole batch"},
            "by_grid_and_batch": table, "gpu_launches": launches, "clocks": clocks.stop(), "e2e": None,
            "cpu_baseline": None}


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.workload in PUNCTURES:
        out = (run_puncture_reference(args, world, rank) if args.impl == "reference"
               else run_puncture(args, world, rank, local))
    elif args.workload == "horizon":
        out = (run_horizon_reference(args, world, rank) if args.impl == "reference"
               else run_horizon(args, world, rank, local))
    elif args.workload in ("adjoint", "batch"):
        if args.impl == "reference":
            why = ("the reference never differentiates its evolution (jax.grad would need JAX, absent here)"
                   if args.workload == "adjoint" else
                   "instance batching has no reference counterpart (its per-instance arm is --workload teukolsky)")
            out = {"impl": "reference", "unavailable": why} if rank == 0 else None
        else:
            out = (run_adjoint if args.workload == "adjoint" else run_batch)(args, world, rank, local)
    elif args.impl == "reference":
        out = run_reference(args, world, rank)
    else:
        out = run_gb300(args, world, rank, local)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
