"""Benchmark: FP64 cell-updates/s of the fused TVD-RK3 path on the 3-D
inviscid Taylor-Green vortex (128^3 periodic on [0, 2 pi]^3, gamma 1.4,
Ma 0.1, WENO5-Z on primitives + HLLC/Einfeldt, RK3, CFL 0.5).

A step is one full TVD-RK3 step (three fused stage kernels + one time-step
kernel) of the whole grid; cell-updates/s = cells x steps / time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``--impl reference`` times the CPU restatement of the reference's algorithm
(the oracle, torch on all host threads) on the same TGV 128^3 workload with
the same warm-up and step counts; the reference itself (JAX) is installed on
neither machine.
Under torchrun each rank advances its own replica (replicas only: the path
has no multi-GPU exchange), and rank 0 prints one JSON line.
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

import torch

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_TGV = 128
METRIC = "FP64 cell-updates/s (TGV 128^3, WENO5-Z+HLLC, TVD-RK3)"
UNIT = "cell-updates/s"
VISCOUS_METRIC = "FP64 cell-updates/s (viscous TGV {n}^3 Re 1600, WENO5-Z CHAR-ROE+HLLC+CENTRAL4, TVD-RK3)"
VISCOUS_SCHEME = "WENO5-Z CHAR-PRIMITIVE (ROE) + HLLC/Einfeldt + CENTRAL4 viscous/heat, TVD-RK3, CFL 0.5"
# Algorithmic HBM bytes per cell-update: stage 1 reads U^n and writes U^1
# (80 B); stages 2 and 3 read U^k and U^n and write (120 B each) -> 320 B.
BYTES_PER_CELL_UPDATE = 320.0
# Algorithmic FP64 operations per cell-update (add, multiply, division and
# square root, one FLOP each): the oracle's count of one RK3 step of the
# reference's algorithm (oracle/flop_count.py; pinned by tests/test_flop_count.py).
FP64_FLOP_ALGORITHMIC = {"tgv": 8280.0, "viscous": 11190.0}
# FP64 thread instructions (DADD + DMUL + DFMA) executed per cell and stage
# by the face kernels of the three axes, from the ncu capture of TGV 128^3 (summary in the
# profiles directory); the epilogue adds the primitives of the new state.
# Viscous CHAR-ROE + HLLC + CENTRAL4: 3 x 1 347.2 per face (viscous TGV 128^3 capture).
FP64_INST_FACES_PER_CELL_STAGE = {"tgv": 2974.8, "viscous": 4041.6}
# DRAM bytes (read + write) of one RK stage at 128^3 from the ncu captures of
# the same build, averaged over the three stages: TGV, the one face launch of
# the three axes (466.7 MB) and the epilogue (579.9 MB); viscous TGV, 473.3 MB
# and 548.9 MB.  Both scale with the cells (the face buffers, the stage
# primitives and the states are per cell); 120 B/cell algorithmic for stages 2, 3.
DRAM_BYTES_PER_STAGE_128 = {"tgv": 1046.6e6, "viscous": 1022.3e6}


def tgv_state(n, device, dtype=torch.float64):
    """Conservatives of the TGV initial condition (interior layout [5, n, n, n])."""
    gamma, ma = 1.4, 0.1
    p0 = 1.0 / (gamma * ma * ma)
    x = (torch.arange(n, dtype=dtype, device=device) + 0.5) * (2 * math.pi / n)
    X, Y, Z = torch.meshgrid(x, x, x, indexing="ij")
    u = torch.sin(X) * torch.cos(Y) * torch.cos(Z)
    v = -torch.cos(X) * torch.sin(Y) * torch.cos(Z)
    w = torch.zeros_like(X)
    p = p0 + (torch.cos(2 * X) + torch.cos(2 * Y)) * (torch.cos(2 * Z) + 2.0) / 16.0
    rho = torch.ones_like(X)
    E = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v + w * w)
    return torch.stack([rho, rho * u, rho * v, rho * w, E]).contiguous()


def tgv_config(n):
    from jaxfluids_gb300 import CaseConfig
    return CaseConfig(cells=(n, n, n), ranges=((0.0, 2 * math.pi),) * 3, nh=3, gamma=1.4,
                      bc={f: "PERIODIC" for f in ("east", "west", "north", "south", "top", "bottom")},
                      recon="WENO5-Z", riemann="HLLC", signal_speed="EINFELDT", cfl=0.5)


def viscous_tgv_config(n):
    """3-D viscous TGV, Re 1600 (mu = 1/1600 with rho0 = U0 = L = 1), Pr 0.71:
    WENO5-Z on Roe-characteristic variables + HLLC + CENTRAL4 dissipative fluxes."""
    from jaxfluids_gb300 import CaseConfig
    return CaseConfig(cells=(n, n, n), ranges=((0.0, 2 * math.pi),) * 3, nh=4, gamma=1.4,
                      bc={f: "PERIODIC" for f in ("east", "west", "north", "south", "top", "bottom")},
                      recon="WENO5-Z", recon_var="CHAR-PRIMITIVE", frozen_state="ROE", riemann="HLLC",
                      signal_speed="EINFELDT", cfl=0.5, viscous=True, heat=True, mu=1.0 / 1600, prandtl=0.71)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[4 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def fp64_peak_tflops(device):
    """DFMA-chain rate of this GPU (8 chains/thread, 152 x 8 CTAs of 256 threads),
    timed with the arithmetic-rate probe library (libgbfprobe.so)."""
    import ctypes
    from jaxfluids_gb300 import build
    lib = ctypes.CDLL(build.build_probe())
    lib.gbf_probe_arith.restype = ctypes.c_int
    lib.gbf_probe_arith.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_void_p]
    blocks, threads, iters = 152 * 8, 256, 2048
    out = torch.empty(blocks * threads, dtype=torch.float64, device=device)
    s = torch.cuda.current_stream()
    st = ctypes.c_void_p(s.cuda_stream)
    lib.gbf_probe_arith(0, ctypes.c_void_p(out.data_ptr()), blocks, threads, 64, st)
    torch.cuda.synchronize()
    best = math.inf
    for _ in range(3):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(s)
        lib.gbf_probe_arith(0, ctypes.c_void_p(out.data_ptr()), blocks, threads, iters, st)
        b.record(s)
        b.synchronize()
        best = min(best, a.elapsed_time(b) / 1e3)
    flops = 2.0 * 8 * iters * blocks * threads
    return flops / best / 1e12


def run_probe(args):
    """The arithmetic-rate probes (libgbfprobe.so): per operation the rate of
    8 independent chains per thread on 152 x 8 CTAs of 256 threads, and its
    cost in DFMA slots.  DDIV_ZERO divides a zero dividend (the division's
    general path, which the kernels' zero-dividend shortcut avoids)."""
    import ctypes
    from jaxfluids_gb300 import build
    device = torch.device("cuda", 0)
    lib = ctypes.CDLL(build.build_probe())
    lib.gbf_probe_arith.restype = ctypes.c_int
    lib.gbf_probe_arith.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_void_p]
    blocks, threads, iters = 152 * 8, 256, 512
    out = torch.empty(blocks * threads, dtype=torch.float64, device=device)
    s = torch.cuda.current_stream()
    st = ctypes.c_void_p(s.cuda_stream)
    rates = {}
    for name, mode in (("dfma", 0), ("ddiv", 1), ("ddiv_zero_dividend", 4), ("dsqrt", 2)):
        lib.gbf_probe_arith(mode, ctypes.c_void_p(out.data_ptr()), blocks, threads, 16, st)
        torch.cuda.synchronize()
        best = math.inf
        for _ in range(3):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(s)
            lib.gbf_probe_arith(mode, ctypes.c_void_p(out.data_ptr()), blocks, threads, iters, st)
            b.record(s)
            b.synchronize()
            best = min(best, a.elapsed_time(b) / 1e3)
        rates[name] = 8.0 * iters * blocks * threads / best
    line = {"metric": "FP64 operation rates (independent chains)", "unit": "G ops/s",
            "value": rates["dfma"] / 1e9, "dtype": "f64", "n_gpus": 1,
            "rates_gops": {k: v / 1e9 for k, v in rates.items()},
            "dfma_slots_per_op": {k: rates["dfma"] / v for k, v in rates.items()}}
    print(json.dumps(line), flush=True)


def cpu_model():
    """CPU model string of this host (lscpu's Model name, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for key in ("Model name:", "Vendor ID:"):
            for line in out.splitlines():
                if line.strip().startswith(key):
                    return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


class OracleRun:
    """The CPU restatement of the reference (oracle, torch float64 on `threads`
    host threads) advancing the TGV n^3 workload step by step: the same
    initial condition, scheme and CFL time step as the GPU run."""

    def __init__(self, n, threads):
        from oracle import jf_oracle as O
        self.O = O
        torch.set_num_threads(threads)
        self.case = O.OracleCase(cells=(n, n, n), ranges=((0.0, 2 * math.pi),) * 3, nh=3,
                                 bc={f: "PERIODIC" for f in O.FACES}, recon="WENO5-Z", riemann="HLLC",
                                 signal_speed="EINFELDT", cfl=0.5)
        U = tgv_state(n, "cpu")
        self.U, self.P = O.initialize(O.prims_from_cons(U, 1.4), self.case)
        self.dt = O.compute_dt(self.P, self.case)
        self.cells = n ** 3

    def step(self):
        """One RK3 step and the next CFL time step; returns its wall time (s)."""
        t0 = time.perf_counter()
        self.U, self.P = self.O.rk3_step(self.U, self.P, self.dt, self.case)
        self.dt = self.O.compute_dt(self.P, self.case)
        return time.perf_counter() - t0


class CPortRun:
    """The plain-C restatement of the reference (oracle/jf_rhs.c, compiled with
    OpenMP on every host core, contraction off; bitwise equal to the torch
    restatement) advancing the TGV n^3 workload step by step: the same initial
    condition, scheme and CFL time step as the GPU run, each face computed
    once per stage as the reference's face arrays hold them.  viscous: the
    viscous TGV's scheme (CHAR-PRIMITIVE with the Roe state, HLLC, CENTRAL4
    viscous and heat fluxes, Re 1600, Pr 0.71) and its dt limits."""

    def __init__(self, n, viscous=False):
        import ctypes
        import __graft_entry__
        from oracle import jf_oracle as O
        so = __graft_entry__.build_oracle_c()
        if not so:
            raise RuntimeError("no C compiler for the oracle's C restatement")
        lib = ctypes.CDLL(so)
        head = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                ctypes.POINTER(ctypes.c_double), ctypes.c_double, ctypes.c_double, ctypes.c_double,
                ctypes.c_double, ctypes.c_int, ctypes.c_int]
        self.U = tgv_state(n, "cpu").numpy().copy()
        self.P = O.prims_from_cons(torch.from_numpy(self.U), 1.4).numpy().copy()
        dx = 2 * math.pi / n
        self.t = ctypes.c_double(0.0)
        self._byref = ctypes.byref
        odx = (ctypes.c_double * 3)(1.0 / dx, 1.0 / dx, 1.0 / dx)
        if viscous:
            cfg = viscous_tgv_config(n)
            f = lib.jf_rk3_steps_visc
            f.argtypes = head + [ctypes.c_double] * 5 + [ctypes.c_int] * 4 + [ctypes.POINTER(ctypes.c_double)]
            cp = cfg.gamma / (cfg.gamma - 1.0) * cfg.R
            self.args = (self.U.ctypes.data, self.P.ctypes.data, (ctypes.c_int * 3)(n, n, n), cfg.nh, odx, dx,
                         cfg.cfl, cfg.gamma, O.STENCIL_EPS, 2, 0,  # CHAR-PRIMITIVE (ROE), HLLC
                         cfg.mu, cfg.bulk_viscosity, cfg.kappa, cp, cfg.R, 1, 1, 1)
        else:
            f = lib.jf_rk3_steps
            f.argtypes = head + [ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
            self.args = (self.U.ctypes.data, self.P.ctypes.data, (ctypes.c_int * 3)(n, n, n), 3, odx, dx, 0.5, 1.4,
                         O.STENCIL_EPS, 0, 0, (ctypes.c_int * 6)(0, 0, 0, 0, 0, 0))  # PRIMITIVE, HLLC, periodic
        f.restype = ctypes.c_int
        self.f = f
        self.cells = n ** 3

    def step(self):
        """One RK3 step (the CFL time step of its initial state); returns its wall time (s)."""
        t0 = time.perf_counter()
        if self.f(*self.args, 1, self._byref(self.t)) != 0:
            raise RuntimeError("the C restatement failed")
        return time.perf_counter() - t0


def cpu_port(n, threads, viscous=False):
    """The fastest CPU restatement available: the C one (OpenMP), else the torch
    one (inviscid TGV only)."""
    try:
        return CPortRun(n, viscous), f"C, OpenMP, {threads} threads"
    except (RuntimeError, OSError):
        if viscous:
            raise
        return OracleRun(n, threads), f"torch float64, {threads} threads"


def run_reference(args, rank, world):
    """The reference arm: the CPU restatement of the reference's algorithm
    (JAX is installed on neither machine, so the reference itself cannot run)
    on the same workload (TGV 128^3, or the viscous TGV 256^3 with
    --workload viscous), all host threads, W warm-up + K timed steps."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    viscous = args.workload == "viscous"
    n = args.n if args.n else (256 if viscous else N_TGV)
    run, how = cpu_port(n, threads, viscous)
    for _ in range(max(0, args.warmup)):
        run.step()
    total_t = sum(run.step() for _ in range(args.steps))
    value = run.cells * args.steps / total_t
    name = "viscous TGV" if viscous else "TGV"
    sample = (f"{name} {n}^3, {args.warmup} warm-up + {args.steps} timed RK3 steps, CPU restatement of the "
              f"reference ({how} on {cpu_model()}); the JAX reference is not installed")
    if viscous:
        metric = VISCOUS_METRIC.format(n=n)
        config = {"workload": f"3-D viscous Taylor-Green vortex {n}^3 periodic, Re 1600, Pr 0.71, Ma 0.1",
                  "cells": n ** 3, "scheme": VISCOUS_SCHEME}
    else:
        metric = METRIC
        config = {"workload": f"3-D inviscid Taylor-Green vortex {n}^3 periodic, Ma 0.1, gamma 1.4",
                  "cells": n ** 3, "scheme": "WENO5-Z PRIMITIVE + HLLC/Einfeldt, TVD-RK3, CFL 0.5"}
    line = {
        "impl": "reference", "metric": metric, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                         "cpu_model": cpu_model()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def batch_cases(ncases=256, seed=0, sides=None):
    """Batched 2-D four-quadrant Riemann problems: sides from {64,...,512}
    (default_rng(0)), or the given sides; per-case quadrant states from
    default_rng(1000 + i): rho, u, v, p drawn per quadrant from U[0.1,2],
    U[-1,1], U[-1,1], U[0.1,2]."""
    import numpy as np
    from jaxfluids_gb300 import CaseConfig
    if sides is None:
        sides = np.random.default_rng(seed).choice([64, 128, 192, 256, 384, 512], size=ncases)
    cfgs, states = [], []
    for i, n in enumerate(sides):
        n = int(n)
        rng = np.random.default_rng(1000 + i)
        st = np.stack([rng.uniform(0.1, 2, 4), rng.uniform(-1, 1, 4), rng.uniform(-1, 1, 4), rng.uniform(0.1, 2, 4)])
        x = (np.arange(n) + 0.5) / n
        X, Y = np.meshgrid(x, x, indexing="ij")
        q = (X >= 0.5).astype(int) + 2 * (Y >= 0.5).astype(int)
        rho, u, v, p = (st[k][q] for k in range(4))
        E = p / 0.4 + 0.5 * rho * (u * u + v * v)
        U = np.stack([rho, rho * u, rho * v, np.zeros_like(rho), E]).reshape(5, n, n, 1)
        cfgs.append(CaseConfig(cells=(n, n, 1), bc={f: "ZEROGRADIENT" for f in ("east", "west", "north", "south")},
                               recon="WENO5-Z", riemann="HLLC", signal_speed="EINFELDT", cfl=0.5))
        states.append(torch.from_numpy(U))
    return cfgs, states


def run_batch(args):
    """Batched (every stage's face and epilogue launches over one work list of
    all cases, graph-captured, autotuned) against one case at a time through
    the single-case fused path."""
    from jaxfluids_gb300 import BatchedRK3, FusedRK3, autotune, build
    build.build()
    device = torch.device("cuda", 0)
    small = args.workload == "batch-small"
    cfgs, states = batch_cases(args.cases, sides=[64] * args.cases if small else None)
    cells = sum(c.n_cells for c in cfgs)
    batch = BatchedRK3(cfgs, device)
    batch.set_states([s.to(device) for s in states])
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    tune = autotune(batch, candidates=[((16, 16, 1), 128, 2 * sms), ((16, 16, 1), 128, 4 * sms),
                                       ((16, 16, 1), 256, 2 * sms), ((16, 8, 1), 128, 4 * sms),
                                       ((32, 16, 1), 256, 2 * sms), ((16, 32, 1), 256, 2 * sms),
                                       ((32, 32, 1), 256, 2 * sms), ((16, 16, 1), 128, 8 * sms)], steps=1)
    graph = batch.capture(args.steps)
    for _ in range(max(1, args.warmup // max(1, args.steps))):
        graph.replay()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    graph.replay()
    b.record()
    b.synchronize()
    t_batch = a.elapsed_time(b) / 1e3
    batched = cells * args.steps / t_batch
    # one case at a time: every case its own fused launches, cases in sequence
    singles = []
    for cfg, s in zip(cfgs, states):
        f = FusedRK3(cfg, device)
        f.set_state(s.to(device))
        singles.append(f)
    for f in singles:
        f.advance(1)
    torch.cuda.synchronize()
    n_single = max(1, min(args.steps, 3))
    a.record()
    for _ in range(n_single):
        for f in singles:
            f.advance(1)
    b.record()
    b.synchronize()
    t_single = a.elapsed_time(b) / 1e3
    single = cells * n_single / t_single
    # one case at a time with each case's steps captured in its own CUDA graph
    # (no host launch overhead; each case still runs alone on the GPU)
    graphs = [f.capture(n_single) for f in singles]
    for g in graphs:
        g.replay()
    torch.cuda.synchronize()
    a.record()
    for g in graphs:
        g.replay()
    b.record()
    b.synchronize()
    t_single_g = a.elapsed_time(b) / 1e3
    single_g = cells * n_single / t_single_g
    mix = "all 64^2" if small else "sides from {64..512}"
    line = {"metric": "FP64 cell-updates/s, batched 2-D four-quadrant Riemann problems", "value": batched,
            "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * t_batch / args.steps, "higher_is_better": True, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": f"{len(cfgs)} cases, {mix}, {cells} cells, WENO5-Z+HLLC, ZG",
                       "autotuned": {"tile": tune["best"][0], "threads": tune["best"][1], "ctas": tune["best"][2]},
                       "graph_steps": args.steps},
            "one_case_at_a_time": {"value": single, "steps": n_single, "ms_per_step": 1e3 * t_single / n_single},
            "one_case_at_a_time_graphs": {"value": single_g, "steps": n_single,
                                          "ms_per_step": 1e3 * t_single_g / n_single},
            "speedup_vs_one_at_a_time": batched / single,
            "speedup_vs_one_at_a_time_graphs": batched / single_g,
            "autotune_ms_per_step": [[list(c[0]), c[1], c[2], ms] for c, ms in tune["results"]]}
    print(json.dumps(line), flush=True)


def kh_state(n, seed, device):
    """2-D Kelvin-Helmholtz on [0,1]^2: rho = 2, u = +0.5 for |y - 0.5| < 0.25,
    else rho = 1, u = -0.5; p = 2.5; v = 0.01 sin(4 pi x) + N(0, 1e-3) noise
    from default_rng(seed).  Returns interior conservatives [5, n, n, 1]."""
    import numpy as np
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x, indexing="ij")
    inner = np.abs(Y - 0.5) < 0.25
    rho = np.where(inner, 2.0, 1.0)
    u = np.where(inner, 0.5, -0.5)
    v = 0.01 * np.sin(4 * np.pi * X) + rng.normal(0.0, 1e-3, X.shape)
    p = np.full_like(X, 2.5)
    E = p / 0.4 + 0.5 * rho * (u * u + v * v)
    U = np.stack([rho, rho * u, rho * v, np.zeros_like(rho), E]).reshape(5, n, n, 1)
    return torch.from_numpy(U).to(device)


def run_dropin(args):
    """The drop-in right-hand side: SpaceSolver.compute_rhs (gbf_rhs_ws, the
    call GB300SpaceSolver's FFI handler makes) on the halo buffers of the TGV
    n^3 state after W fused warm-up steps (not the symmetric initial state),
    K calls timed with CUDA events, L2 overwritten between calls; beside it a
    fused stage (one third of a fused step) on the same state."""
    from jaxfluids_gb300 import FusedRK3, SpaceSolver, build
    from jaxfluids_gb300.solver import EquationManager, HaloManager
    build.build()
    device = torch.device("cuda", 0)
    n = args.n if args.n else N_TGV
    cfg = tgv_config(n)
    f = FusedRK3(cfg, device)
    f.set_state(tgv_state(n, device))
    f.advance(max(3, args.warmup))
    U0 = f.cons.clone()
    hs = cfg.halo_shape()
    inner = (slice(None),) + tuple(slice(cfg.nh, cfg.nh + n) for _ in range(3))
    Uh = torch.zeros(hs, dtype=torch.float64, device=device)
    Ph = torch.zeros(hs, dtype=torch.float64, device=device)
    Uh[inner] = U0
    Ph[inner] = EquationManager(cfg).get_primitives_from_conservatives(U0.contiguous())
    Ph, Uh = HaloManager(cfg).perform_halo_update_material(Ph, 0.0, conservatives=Uh)
    solver = SpaceSolver(cfg)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    for _ in range(3):
        solver.compute_rhs(Uh, Ph, None, 0.0, 0.0)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for k, (a, b) in enumerate(ev):
        flush.fill_(float(k))
        a.record()
        solver.compute_rhs(Uh, Ph, None, 0.0, 0.0)
        b.record()
    torch.cuda.synchronize()
    t_rhs = sum(a.elapsed_time(b) for a, b in ev) / 1e3 / args.steps
    fev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for k, (a, b) in enumerate(fev):
        flush.fill_(float(k))
        a.record()
        f.advance(1)
        b.record()
    torch.cuda.synchronize()
    t_stage = sum(a.elapsed_time(b) for a, b in fev) / 1e3 / args.steps / 3.0
    cells = n ** 3
    line = {"metric": f"FP64 cell right-hand sides/s (drop-in compute_rhs, TGV {n}^3, WENO5-Z+HLLC)",
            "value": cells / t_rhs, "unit": "cells/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_rhs": 1e3 * t_rhs, "higher_is_better": True, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"TGV {n}^3 after {max(3, args.warmup)} fused steps, halo buffers filled by "
                                   "the halo update", "entry": "SpaceSolver.compute_rhs -> gbf_rhs_ws",
                       "l2": "256 MiB buffer written between timed calls"},
            "fused_stage_ms": 1e3 * t_stage, "rhs_over_fused_stage": t_rhs / t_stage,
            "gpu_launches": 2 * args.steps}
    print(json.dumps(line), flush=True)


def run_adjoint(args):
    """Gradient of 1/2 ||rho(T) - rho_target||^2 w.r.t. the initial state through
    args.adj_steps fixed-dt RK3 steps (dt = CFL 0.5 step of the initial state),
    checkpoints every 50 steps; cost relative to the plain forward run."""
    from jaxfluids_gb300 import CaseConfig, FusedRK3, build
    from jaxfluids_gb300.adjoint import AdjointRK3
    build.build()
    device = torch.device("cuda", 0)
    n = args.adj_n
    cfg = CaseConfig(cells=(n, n, 1), bc={f: "PERIODIC" for f in ("east", "west", "north", "south")},
                     recon="WENO5-Z", riemann="HLLC", signal_speed="EINFELDT", cfl=0.5)
    U0 = kh_state(n, 7, device)
    f = FusedRK3(cfg, device)
    f.set_state(U0)
    dt = float(f.dt)
    adj = AdjointRK3(cfg, dt, device)
    target = adj.advance(kh_state(n, 8, device), args.adj_steps)[0]
    steps = args.adj_steps
    adj.advance(U0, 5)  # warm-up
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    UN = adj.advance(U0, steps)
    b.record()
    b.synchronize()
    t_fwd = a.elapsed_time(b) / 1e3
    adj.forward_steps = 0
    a.record()
    UN2, grad = adj.gradient(U0, steps, lambda U: torch.stack([U[0] - target] + [torch.zeros_like(target)] * 4),
                             schedule=args.adj_schedule, every=args.adj_every)
    b.record()
    b.synchronize()
    t_adj = a.elapsed_time(b) / 1e3
    # gradient w.r.t. the initial v field: U = cons(P), d(rho v)/dv = rho, dE/dv = rho v
    rho0 = U0[0]
    dv = grad[2] * rho0 + grad[4] * U0[2]
    line = {"metric": "adjoint cost / forward cost, 2-D Kelvin-Helmholtz", "value": t_adj / t_fwd,
            "unit": "x", "higher_is_better": False, "n_gpus": 1, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"KH {n}^2 periodic, {steps} fixed-dt RK3 steps (dt {dt:.4e})",
                       "schedule": args.adj_schedule, "checkpoint_every": args.adj_every, "cells": n * n},
            "forward_s": t_fwd, "gradient_s": t_adj, "forward_steps_recomputed": adj.forward_steps,
            # the gradient's two parts: the forward run that places the
            # checkpoints, and the reverse sweep (replays + step VJPs)
            "gradient_forward_s": adj.last_split[0], "gradient_reverse_s": adj.last_split[1],
            "reverse_over_forward": adj.last_split[1] / t_fwd,
            "forward_cell_updates_per_s": n * n * steps / t_fwd,
            "grad_v_norm": float(dv.norm()), "loss": float(0.5 * ((UN[0] - target) ** 2).sum())}
    print(json.dumps(line), flush=True)


def run_viscous_adjoint(args):
    """Adjoint of the viscous TGV (CHAR-ROE + HLLC + CENTRAL4, Re 1600, Pr 0.71):
    gradient of the final kinetic energy w.r.t. the initial velocity over a
    fixed-dt trajectory, reversed with binomial checkpoints whose segments of
    up to `leaf` steps are replayed keeping their stage states.  Reports the cost
    of the gradient (forward for the loss + recomputation + reverse sweep)
    over the cost of the forward run alone."""
    from jaxfluids_gb300 import FusedRK3, build
    from jaxfluids_gb300.adjoint import AdjointRK3
    build.build()
    device = torch.device("cuda", 0)
    n = args.n if args.n else 256
    cfg = viscous_tgv_config(n)
    U0 = tgv_state(n, device)
    f = FusedRK3(cfg, device)
    f.set_state(U0)
    dt = float(f.dt)
    del f
    adj = AdjointRK3(cfg, dt, device)
    steps = args.adj_steps
    adj.advance(U0, 2)  # warm-up
    torch.cuda.synchronize()

    def ke_grad(U):
        # KE = sum (rho u)^2 / (2 rho): dKE/d(rho u_i) = u_i, dKE/drho = -|u|^2 / 2
        u = U[1:4] / U[0]
        return torch.cat([(-0.5 * (u * u).sum(0))[None], u, torch.zeros_like(U[:1])])

    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    UN = adj.advance(U0, steps)
    b.record()
    b.synchronize()
    t_fwd = a.elapsed_time(b) / 1e3
    del UN
    adj.forward_steps = 0
    torch.cuda.reset_peak_memory_stats(device)
    a.record()
    UN2, grad = adj.gradient(U0, steps, ke_grad, schedule="binomial", slots=args.adj_slots, leaf=args.adj_leaf)
    b.record()
    b.synchronize()
    t_adj = a.elapsed_time(b) / 1e3
    rho0 = U0[0]
    gu = torch.stack([grad[1 + i] * rho0 + grad[4] * U0[1 + i] for i in range(3)])
    ke = float((0.5 * (UN2[1:4] ** 2).sum(0) / UN2[0]).sum())
    line = {"metric": "adjoint cost / forward cost, 3-D viscous TGV", "value": t_adj / t_fwd, "unit": "x",
            "higher_is_better": False, "n_gpus": 1, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"viscous TGV {n}^3 Re 1600 Pr 0.71, CHAR-ROE WENO5-Z + HLLC + CENTRAL4, "
                                   f"{steps} fixed-dt RK3 steps (dt {dt:.4e})",
                       "schedule": "binomial", "slots": args.adj_slots, "leaf": args.adj_leaf,
                       "cells": n ** 3},
            "forward_s": t_fwd, "gradient_s": t_adj, "forward_steps_recomputed": adj.forward_steps,
            "gradient_forward_s": adj.last_split[0], "gradient_reverse_s": adj.last_split[1],
            "reverse_over_forward": adj.last_split[1] / t_fwd,
            "peak_device_gb": torch.cuda.max_memory_allocated(device) / 1e9,
            "final_ke": ke, "grad_u_norm": float(gu.norm())}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=None, help="grid side (default 128 inviscid, 256 viscous)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="tgv",
                    choices=["tgv", "viscous", "batch", "batch-small", "adjoint", "viscous-adjoint", "dropin",
                             "probe"])
    ap.add_argument("--adj-n", type=int, default=512)
    ap.add_argument("--adj-steps", type=int, default=None, help="default 1000 (KH), 200 (viscous TGV)")
    ap.add_argument("--adj-slots", type=int, default=2, help="binomial checkpoint slots (viscous adjoint)")
    ap.add_argument("--adj-leaf", type=int, default=100,
                    help="binomial: longest segment replayed once with its stage states kept (viscous adjoint)")
    ap.add_argument("--adj-every", type=int, default=50)
    ap.add_argument("--adj-schedule", default="stored", choices=["stored", "uniform", "binomial"])
    ap.add_argument("--cases", type=int, default=256)
    args = ap.parse_args()
    if args.workload in ("batch", "batch-small"):
        return run_batch(args)
    if args.workload == "adjoint":
        args.adj_steps = args.adj_steps or 1000
        return run_adjoint(args)
    if args.workload == "dropin":
        return run_dropin(args)
    if args.workload == "probe":
        return run_probe(args)
    if args.workload == "viscous-adjoint":
        args.adj_steps = args.adj_steps or 200
        return run_viscous_adjoint(args)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import ctypes
    from jaxfluids_gb300 import FusedRK3, _lib, build
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    if rank == 0:
        build.build()
    if world > 1:
        dist.barrier()
    lib = _lib.load()
    viscous = args.workload == "viscous"
    n = args.n if args.n else (256 if viscous else N_TGV)
    cfg = viscous_tgv_config(n) if viscous else tgv_config(n)
    cells = n ** 3
    U0 = tgv_state(n, device)
    f = FusedRK3(cfg, device)
    f.set_state(U0)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    stream = torch.cuda.current_stream()

    for _ in range(args.warmup):
        f.advance(1)
    torch.cuda.synchronize()

    sampler = ClockSampler(local)
    sampler.start()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    t_wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.fill_(float(k))          # overwrite L2 (256 MiB > 129 MB) between steps
        starts[k].record(stream)
        f.advance(1)
        ends[k].record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    wall = time.perf_counter() - t_wall0
    clocks = sampler.stop()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    t_dev = sum(step_ms) / 1e3
    if world > 1:
        tt = torch.tensor([t_dev], device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_dev = tt.item()
    value = world * cells * args.steps / t_dev

    # ---- per-stage time (face kernel + epilogue; same stream, CUDA events) ----
    ka = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    kb = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    for k in range(3):
        ka[k].record(stream)
        f.advance(1)
        kb[k].record(stream)
    torch.cuda.synchronize()
    per_step_s = min(a.elapsed_time(b) for a, b in zip(ka, kb)) / 1e3
    # a step = 3 stages (+ the primitives of U^n and the one-thread time-step
    # kernel, ~0.2 % of the step)
    stage_s = per_step_s / 3.0
    bytes_per_stage = BYTES_PER_CELL_UPDATE / 3.0 * cells
    hbm_peak, peak_src = 6800.0, "fallback (6.8 TB/s)"
    try:
        hbm_peak = float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"])
        peak_src = "measured"
    except Exception:
        pass
    achieved = bytes_per_stage / stage_s / 1e9
    fp64_peak = fp64_peak_tflops(device)
    kind = "viscous" if viscous else "tgv"
    flop_alg = FP64_FLOP_ALGORITHMIC[kind]
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
        "frac": achieved / hbm_peak, "peak_source": peak_src,
        "traffic": DRAM_BYTES_PER_STAGE_128[kind] * cells / 128 ** 3,
        "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one stage at 128^3"
                          + ("" if n == 128 else f", scaled by the cells to {n}^3"),
        "launch": "one RK stage: face_flux_kernel (x, y, z faces) + stage_epilogue_kernel",
        "fp64": {
            "peak_tflops_measured": fp64_peak,  # DFMA chains, 2 FLOP per instruction
            "flop_per_cell_update_algorithmic": flop_alg,
            "achieved_tflops_algorithmic": flop_alg * cells / per_step_s / 1e12,
            "frac_algorithmic": flop_alg * cells / per_step_s / 1e12 / fp64_peak,
            "inst_per_cell_stage_faces": FP64_INST_FACES_PER_CELL_STAGE[kind],
            "frac_issue_faces": FP64_INST_FACES_PER_CELL_STAGE[kind] * cells / stage_s / (fp64_peak * 1e12 / 2.0),
        },
    }

    # ---- end to end through the public API with host buffers ----
    # A host-driven time loop: the state lives in pinned host memory; every
    # step copies it to the device, advances it one step through the public
    # API and copies the result back (the next step's input), so the state
    # evolves as in the device-resident loop above.
    host = torch.empty((5, n, n, n), dtype=torch.float64, pin_memory=True)
    host.copy_(f.cons.view(5, n, n, n))
    e2e_steps = max(3, min(args.steps, 10))
    torch.cuda.synchronize()
    ea = torch.cuda.Event(enable_timing=True)
    eb = torch.cuda.Event(enable_timing=True)
    ea.record(stream)
    for _ in range(e2e_steps):
        f.cons.copy_(host.view(f.cons.shape), non_blocking=True)
        f.advance(1)
        host.view(f.cons.shape).copy_(f.cons, non_blocking=True)
    eb.record(stream)
    torch.cuda.synchronize()
    e2e_t = ea.elapsed_time(eb) / 1e3
    e2e = {"value": world * cells * e2e_steps / e2e_t, "unit": UNIT,
           "h2d_bytes_per_step": host.numel() * 8, "d2h_bytes_per_step": host.numel() * 8,
           "steps": e2e_steps}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        run, how = cpu_port(n, threads, viscous)
        run.step()  # warm-up
        el = sum(run.step() for _ in range(3))
        cpu = {"value": run.cells * 3 / el, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{'viscous ' if viscous else ''}TGV {n}^3 (the same workload), 1 warm-up + 3 timed RK3 "
                         f"steps ({el:.1f} s), CPU restatement of the reference ({how})",
               "cpu_model": cpu_model()}

    if rank == 0:
        metric = METRIC if not viscous else VISCOUS_METRIC.format(n=n)
        line = {
            "metric": metric, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": (f"3-D viscous Taylor-Green vortex {n}^3 periodic, Re 1600, Pr 0.71, Ma 0.1"
                                    if viscous else f"3-D inviscid Taylor-Green vortex {n}^3 periodic, Ma 0.1, gamma 1.4"),
                       "cells": cells,
                       "scheme": (VISCOUS_SCHEME if viscous else "WENO5-Z PRIMITIVE + HLLC/Einfeldt, TVD-RK3, CFL 0.5"),
                       "parallelism": f"replicas x{world}",
                       "l2": "256 MiB buffer written between timed steps (per-step CUDA events)"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            # per advance(1): the stage primitives of U^n, three stages of one face
            # kernel per axis and one epilogue, the time-step kernel
            # per step: the primitives of U^n (convert_kernel), per stage one
            # face-kernel launch (every axis) and the epilogue, the next dt
            "gpu_launches": (1 + 3 * (1 + 1) + 1) * args.steps, "clocks": clocks, "wall_s": wall,
            "step_ms": {"min": min(step_ms), "median": statistics.median(step_ms), "max": max(step_ms)},
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
