#!/usr/bin/env python
"""Throughput of the batched PNJL gap solve on one GB300 (bench contract of this repository).

Workload (default ``--workload first_order_2048x2048x9``, the largest single-GPU
configuration): the first-order-region scan T = linspace(20, 150, 2048) MeV x
mu_u = linspace(250, 450, 2048) MeV, mu_s = mu_u / 2, x xi in {-0.4, ..., 0.4} (37,748,736
points), 128 momentum x 32 cos(theta) Gauss-Legendre nodes, 8 seed candidates (MultiSeed +
MEDIUM, HIGH_DENSITY) with global-min-Omega selection, converged when
||grad_x Omega||_inf < 1e-10.  A "step" solves one strided slice of the grid (every
n_chunks-th point, 18,432 points, a different slice each step), so the timed steps are spread
over the whole (T, mu, xi) box; the slices are decoded from the flat index when loaded.
Inputs (T, mu, xi) are synthetic grid points: there is no dataset.  Other workloads:
``aniso_scan_256x256x9`` (T 50-300 MeV x mu 0-400 MeV x 9 xi, 589,824 points, 4 seeds),
``surrogate_eval_2p20`` (2^20 uniform points, MultiSeed (6)) and ``iso_scan_32x32``.

Headline (``--mode surrogate``): surrogate-seeded mixed-precision solves -- the trained
network's seed per point (BF16 tensor-core inference kernel), one mixed-precision Newton solve
(FP32 Kahan node passes, FP64 solve/update/residual), verification by every seed candidate
where a second phase can exist (the cells of the network's verification map, roots far from
the seed, roots on an unstable branch), MultiSeed fallback where the learned seed fails.  The
network is trained in an untimed set-up on this GPU (labels: a 64 x 64 x 5 (T, mu, xi)
multi-seed solve over the workload's box; 300 epochs), reported as ``surrogate.train``, and
``surrogate.amortised`` is the whole grid's rate with that set-up included.  The same chunks
are then solved by the plain FP64 multi-seed Newton (the workload's candidates, min-Omega
selection, trust-region fallback): ``plain_fp64`` holds its rate, the speed-up, and the phase
misassignments of the surrogate path against it.  ``parity`` checks both arms' roots against
the oracle's (root to rounding; phase from its MultiSeed solve) on the points where the arms
disagree and on uniformly drawn points.  ``--mode multiseed --precision fp64|mixed`` times
the MultiSeed table path alone; ``--mode orders`` the 32 x 32 grid at three quadrature orders
in one graph.

value: converged solves per second with inputs already in HBM (pnjl_solve_batch_learned_device
or pnjl_solve_batch_device), timed with CUDA events on the library's stream; e2e: the same
metric through the host-array entry point (pnjl_solve_batch_learned / pnjl_solve_batch),
pinned host inputs, host<->device copies inside the timed region.  roofline: the dominant
kernel's algorithmic FP64, FP32 and SFU (MUFU) rates against pipe peaks measured in the run.
``--impl reference`` times the reference algorithm's CPU restatement (the oracle: nested
forward-mode derivatives like the reference's ForwardDiff, NLsolve-style Newton, MultiSeed
min-Omega) on a bounded sample of the same workload with all host threads.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

HBARC = 197.327
# DRAM bytes (read + write) per launch of the dominant kernel from one ncu capture of a
# 9,216-point launch (0.058 GB + 0.274 GB), scaled by points to the 18,432-point step; it is
# mostly local-memory (stack) write-back (inputs and outputs are 240 B per point)
TRAFFIC = {"mixed_fused_kernel<32>": {
    "bytes_per_launch": 2 * (0.057730048e9 + 0.273578240e9),
    "source": "ncu --set full of one 9,216-point launch (profiles/mixed_fused_kernel_surrogate_aniso_9216pt.md), "
              "scaled by points; mostly local-memory write-back"}}
METRIC = "gap solves/s at \u2016\u2202\u03a9\u2016\u22641e-10: surrogate-seeded vs plain FP64 Newton, 1 GB300"
# Floating-point operations per node-flavour evaluation, counted from the source of
# pnjl_device.cuh::node_flavour (FMA = 2, loop invariants hoisted, selects and compares not
# counted; the transcendental calls -- rsqrt, exp, rcp, and log in thermo passes -- are
# counted separately and not as FLOPs):
#   Newton pass (residual + Jacobian):        123 FLOP + 3 transcendentals
#   thermo pass (Omega, s, rho, n_f at the end): 58 FLOP + 4 transcendentals
#   residual-only pass (mixed-precision refinement):  53 FLOP + 3 transcendentals
#   residual + thermo pass (mixed refinement):        69 FLOP + 4 transcendentals
#   FP32 Newton pass: 123 FLOP + 27 for the Kahan compensation of 9 sums = 150 FLOP
#   FP32 Omega pass (candidate pruning): 58 FLOP + 6 for 2 compensated sums = 64 FLOP
#   float-float residual pass: the 53 residual FLOP, float-float thermo pass: the 58 thermo
#     FLOP, each a float-float operation of 6-20 FP32 instructions; reported as their own
#     count, not added to the FP32 FLOP
FLOP_NEWTON = 123
FLOP_THERMO = 58
FLOP_GRAD = 53
FLOP_GRAD_THERMO = 69
FLOP_NEWTON32 = 150
FLOP_THERMO32 = 64
FLOP_FF = 53
FLOP_FF_THERMO = 58
# SFU (MUFU) operations per node-flavour evaluation, counted from the pass sources:
#   FP32 Newton pass (node_pass_newton32): rsqrt, ex2 (__expf), 2 rcp.approx       = 4
#   FP32 Omega pass: rsqrt, ex2, rcp, lg2 (__logf)                                   = 4
#   float-float passes (pnjl_ff.cuh): rsqrt seed of ff_rsqrt, 2 rcp.approx seeds of
#     ff_rcp (ff_exp and ff_log are table methods: no MUFU)                          = 3
#   FP64 certification pass (node_pass_cert): rsqrt.approx.f64, rcp.approx.f64
#     (its exp is a table method)                                                    = 2
#   plain FP64 passes: the seeds of the library's double rsqrt and 1/x               = 2
MUFU = {"node_evals_fp32": 4, "node_evals_fp32_thermo": 4, "node_evals_ff": 3, "node_evals_ff_thermo": 3,
        "node_evals_ff_grad_thermo": 3, "node_evals_fp64_grad": 2, "node_evals_fp64_grad_thermo": 2,
        "node_evals_fp64_newton": 2, "node_evals_fp64_thermo": 2}


def pass_mufu(st: dict) -> float:
    """SFU (MUFU) operations of one solve from the node-evaluation counters."""
    return float(sum(st[k] * v for k, v in MUFU.items()))


def pass_flops(st: dict):
    """(FP64 FLOP, FP32 FLOP, float-float FLOP) of one solve from the node-evaluation counters."""
    f64 = (st["node_evals_fp64_newton"] * FLOP_NEWTON + st["node_evals_fp64_thermo"] * FLOP_THERMO +
           st["node_evals_fp64_grad"] * FLOP_GRAD + st["node_evals_fp64_grad_thermo"] * FLOP_GRAD_THERMO)
    f32 = st["node_evals_fp32"] * FLOP_NEWTON32 + st["node_evals_fp32_thermo"] * FLOP_THERMO32
    return f64, f32, (st["node_evals_ff"] * FLOP_FF + st["node_evals_ff_thermo"] * FLOP_FF_THERMO +
                      st["node_evals_ff_grad_thermo"] * FLOP_GRAD_THERMO)


XI9 = np.round(np.arange(-0.4, 0.4001, 0.1), 10)  # -0.4, -0.3, ..., 0.4


def stored_grid(T, mu_u, mu_s, xi, **kw):
    """A workload held as arrays (T, mu in fm^-1); at(idx) -> (T, mu_u, mu_s, xi)."""
    return dict(n=T.size, at=lambda idx: (T[idx], mu_u[idx], mu_s[idx], xi[idx]), **kw)


def workload_grid(name: str):
    """The bench workloads: points (T, mu_u = mu_d, mu_s, xi), node counts, seed table and,
    for the surrogate arm, the network's training box."""
    from julia_relaxtime_gb300 import pnjl
    from julia_relaxtime_gb300.learned_seed import TrainConfig

    if name == "aniso_scan_256x256x9":
        T = np.linspace(50.0, 300.0, 256)
        mu = np.linspace(0.0, 400.0, 256)
        Tg, mg, xg = np.meshgrid(T, mu, XI9, indexing="ij")
        mu = mg.ravel() / HBARC
        return stored_grid(Tg.ravel() / HBARC, mu, mu, xg.ravel().copy(), p_num=128, t_num=32, n_seeds=4, extra=(),
                           chunks=32, train=TrainConfig(),
                           desc="256x256 (T 50-300 MeV, mu 0-400 MeV) x 9 xi, p128 x t32, 4 seeds, min-Omega")
    if name == "iso_scan_32x32":
        T = np.linspace(50.0, 300.0, 32)
        mu = np.linspace(0.0, 400.0, 32)
        Tg, mg = np.meshgrid(T, mu, indexing="ij")
        n = Tg.size
        mu = mg.ravel() / HBARC
        return stored_grid(Tg.ravel() / HBARC, mu, mu, np.zeros(n), p_num=64, t_num=8, n_seeds=6, extra=(), chunks=1,
                           train=TrainConfig(),
                           desc="32x32 (T 50-300 MeV, mu 0-400 MeV), xi = 0, p64 x t8, MultiSeed (6), min-Omega")
    if name == "surrogate_eval_2p20":
        # 2^20 points uniform in the training box, from a counter-based generator (Philox, key
        # 20240611): the same points on every machine and numpy version
        rng = np.random.Generator(np.random.Philox(key=20240611))
        n = 1 << 20
        T = rng.uniform(50.0, 300.0, n) / HBARC
        mu = rng.uniform(0.0, 400.0, n) / HBARC
        xi = rng.uniform(-0.5, 0.5, n)
        return stored_grid(T, mu, mu, xi, p_num=128, t_num=32, n_seeds=6, extra=(), chunks=32, train=TrainConfig(),
                           desc="2^20 points U[50,300] MeV x U[0,400] MeV x U[-0.5,0.5] (Philox key 20240611), "
                                "p128 x t32, MultiSeed (6), min-Omega")
    if name == "first_order_2048x2048x9":
        # 37,748,736 points, decoded from the flat index (T slowest, xi fastest) when a slice
        # is loaded; mu_s = 0.5 mu_u
        nT = nm = 2048
        Tv = np.linspace(20.0, 150.0, nT) / HBARC
        mv = np.linspace(250.0, 450.0, nm) / HBARC

        def at(idx):
            idx = np.asarray(idx, dtype=np.int64)
            ix = idx % XI9.size
            r = idx // XI9.size
            mu_u = mv[r % nm]
            return Tv[r // nm], mu_u, 0.5 * mu_u, XI9[ix]

        extra = (pnjl.MEDIUM_SEED_5, pnjl.HIGH_DENSITY_SEED_5)
        return dict(n=nT * nm * XI9.size, at=at, p_num=128, t_num=32, n_seeds=6, extra=extra, chunks=2048,
                    train=TrainConfig(T_MeV=(20.0, 150.0, 64), mu_MeV=(250.0, 450.0, 64), xi=(-0.5, 0.5, 5),
                                      mu_s_ratio=0.5, label_seeds=6, label_extra=extra),
                    desc="2048x2048 (T 20-150 MeV, mu_u 250-450 MeV, mu_s = mu_u/2) x 9 xi, p128 x t32, "
                         "8 seeds (MultiSeed + MEDIUM, HIGH_DENSITY), min-Omega")
    raise SystemExit(f"unknown workload {name}")


def slice_indices(n: int, rank: int, world: int, chunks: int, c: int) -> np.ndarray:
    """Global indices of slice c (mod chunks) of rank's shard: shard_points(n, rank, world)[c::chunks],
    computed without materialising the shard."""
    n_local = len(range(rank, n, world))
    return rank + world * np.arange(c % chunks, n_local, chunks, dtype=np.int64)


def seed_count(grid) -> int:
    return grid["n_seeds"] + len(grid["extra"])


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def run_reference(args, grid, sample_points: int, threads: int | None = None):
    """The reference algorithm on the CPU (oracle restatement), bounded sample, all threads
    (or `threads`)."""
    from oracle import oracle as orc

    P = orc.default_params()
    nd = orc.Nodes(grid["p_num"], grid["t_num"])
    threads = threads or os.cpu_count() or 1
    n = grid["n"]
    rng = np.random.default_rng(1234)
    idx = np.sort(rng.choice(n, size=min(sample_points, n), replace=False))
    opts = orc.default_opts(max_iter=40, ftol=1e-10)
    T, mu_u, mu_s, xi = grid["at"](idx)
    mu3 = np.stack([mu_u, mu_u, mu_s], axis=1)
    kw = dict(n_seeds=grid["n_seeds"])
    if grid["extra"]:
        # an explicit candidate table: the MultiSeed candidates below T = 300 MeV plus the extra
        # rows (the workloads with extra rows lie below 300 MeV, where the table is fixed)
        from julia_relaxtime_gb300.pnjl import multiseed_table

        assert float(np.max(T)) * HBARC < 300.0
        kw = dict(seeds=multiseed_table(grid["n_seeds"], grid["extra"])[0], multiseed_rule=False)
    times, solved = [], 0
    for it in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        rs = orc.solve_batch(P, nd, T, mu3, xi, multi=True, opts=opts, threads=threads, **kw)
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            times.append(dt)
            solved += sum(1 for r in rs if r.converged and r.residual_norm <= 1e-10)
    total = sum(times)
    return dict(value=solved / total, seconds=total, cores=threads, points=len(idx),
                sample=f"{len(idx)} points drawn uniformly (seed 1234) from the workload grid, per step")


def single_thread_rate(grid, sample_points: int) -> dict:
    """The same CPU restatement on one thread, over a few of the same points (one pass)."""
    class A:  # noqa: N801
        warmup, steps = 0, 1
    r = run_reference(A, grid, sample_points, threads=1)
    return {"value": r["value"], "unit": "solves/s", "cores": 1, "sample": r["sample"]}


def parity_vs_oracle(grid, arms: dict, chunk_points, n_uniform: int = 2000, n_phase: int = 384, seed: int = 4321):
    """The timed arms' roots against the oracle (CPU, FP64 nested-jet Newton: the reference
    algorithm), on the points where the arms disagree by more than 1e-9 (relative, per
    condensate) plus n_uniform points drawn from the timed slices.

    Reference root: the oracle's plain Newton at ftol 1e-13 (no step test) from the plain
    FP64 arm's root -- the root to rounding (oracle.polish).  Phase: the oracle's MultiSeed
    min-Omega solve at the bench's ftol on n_phase of the uniform points.  Per arm:
    |dphi|_inf / |phi|_inf (the condensate vector), |dPhi|_inf (Phi, Phibar), |dOmega|/|Omega|."""
    from oracle import oracle as orc

    t0 = time.perf_counter()
    names = list(arms)
    pts, cols = [], {a: {"x": [], "omega": [], "ok": []} for a in names}
    for k, rr in enumerate(arms[names[0]]):
        T, mu_u, mu_s, xi = chunk_points(rr["chunk"])
        pts.append(np.stack([T, mu_u, mu_s, xi], axis=1))
        for a in names:
            r = arms[a][k]
            cols[a]["x"].append(r["x"])
            cols[a]["omega"].append(r["omega"])
            cols[a]["ok"].append(r["converged"])
    pts = np.concatenate(pts)
    X = {a: np.concatenate(cols[a]["x"]) for a in names}
    OM = {a: np.concatenate(cols[a]["omega"]) for a in names}
    ok = np.logical_and.reduce([np.concatenate(cols[a]["ok"]) for a in names])
    a0, a1 = names
    rel = np.abs(X[a0][:, :3] - X[a1][:, :3]) / np.maximum(np.abs(X[a1][:, :3]), 1e-300)
    flagged = np.flatnonzero(ok & (rel.max(axis=1) > 1e-9))
    rng = np.random.default_rng(seed)
    rest = np.setdiff1d(np.flatnonzero(ok), flagged)
    uni = np.sort(rng.choice(rest, size=min(n_uniform, rest.size), replace=False))
    sel = np.concatenate([flagged, uni])
    P = orc.default_params()
    nd = orc.Nodes(grid["p_num"], grid["t_num"])
    T, mu_u, mu_s, xi = (pts[sel, j].copy() for j in range(4))
    mu3 = np.stack([mu_u, mu_u, mu_s], axis=1)
    threads = os.cpu_count() or 1
    xt, omt, rt = orc.polish(P, nd, T, mu3, xi, X["plain_fp64"][sel], threads=threads)
    out = {"reference": "oracle root to rounding: plain Newton at ftol 1e-13 from the plain FP64 arm's root "
                        "(oracle.polish); phase from the oracle's MultiSeed min-Omega solve (ftol 1e-10)",
           "points": int(sel.size), "points_arms_differ_above_1e-9": int(flagged.size), "points_uniform": int(uni.size),
           "bound": {"dphi_over_phi_inf": 1e-9, "dPhi_abs": 1e-10},
           "oracle_residual_max": float(np.max(rt))}
    phi_scale = np.abs(xt[:, :3]).max(axis=1)
    for a in names:
        x, om = X[a][sel], OM[a][sel]
        dphi = np.abs(x[:, :3] - xt[:, :3]).max(axis=1) / phi_scale
        dPhi = np.abs(x[:, 3:] - xt[:, 3:]).max(axis=1)
        dom = np.abs(om - omt) / np.abs(omt)
        out[a] = {"max_dphi_over_phi": float(dphi.max()), "points_dphi_above_1e-9": int(np.sum(dphi > 1e-9)),
                  "max_abs_dPhi": float(dPhi.max()), "points_dPhi_above_1e-10": int(np.sum(dPhi > 1e-10)),
                  "max_rel_domega": float(dom.max())}
    # phase selection against the oracle's own MultiSeed solve
    ph = uni[:min(n_phase, uni.size)]
    T, mu_u, mu_s, xi = (pts[ph, j].copy() for j in range(4))
    mu3 = np.stack([mu_u, mu_u, mu_s], axis=1)
    kw = dict(n_seeds=grid["n_seeds"])
    if grid["extra"]:
        from julia_relaxtime_gb300.pnjl import multiseed_table

        kw = dict(seeds=multiseed_table(grid["n_seeds"], grid["extra"])[0], multiseed_rule=False)
    rs = orc.solve_batch(P, nd, T, mu3, xi, multi=True, opts=orc.default_opts(max_iter=40, ftol=1e-10),
                         threads=threads, **kw)
    om_o = np.array([r.omega for r in rs])
    conv_o = np.array([bool(r.converged) for r in rs])
    out["phase_check"] = {"points": int(ph.size), "oracle_converged": int(conv_o.sum())}
    for a in names:
        diff = np.abs(OM[a][ph] - om_o) > 1e-10 * np.abs(om_o)
        out["phase_check"][f"misassignments_{a}"] = int(np.sum(diff & conv_o))
    out["seconds"] = time.perf_counter() - t0
    out["threads"] = threads
    return out


class Arm:
    """One solve configuration timed over the same strided chunks of the grid."""

    def __init__(self, name, eng, table, hot, opts, learned):
        self.name, self.eng, self.table, self.hot, self.opts, self.learned = name, eng, table, hot, opts, learned

    def launch(self, n, d_in, ptrs):
        m = d_in["mu"].data_ptr()
        self.eng.solve_device(n, d_in["T"].data_ptr(), m, m, d_in["mu_s"].data_ptr(), d_in["xi"].data_ptr(), ptrs,
                              seed_table=self.table,
                              seed_table_hot=self.hot, opts=self.opts, learned=self.learned)


def run_scan(args):
    """The drop-in scan driver end to end: scan.run_gap_transport_scan (the gap part of
    scripts/relaxtime/run_gap_transport_scan.jl) over T 50-300 MeV x mu_B 0-1200 MeV (32 x 32,
    mu_q = mu_B / 3: the 32 x 32 isotropic grid's box) x xi in {0, 0.2, 0.4}, p64 x t8,
    MultiSeed on each (xi, mu_B) column's first point and PhaseAwareContinuitySeed after it
    (the reference's boundary.csv / cep.csv), build_K_data per row, CSV written.  Timed on the
    host clock around the whole driver (trackers, launches, copies, CSV); the same driver over
    the oracle on all host cores beside it."""
    import tempfile

    from julia_relaxtime_gb300.engine import GapEngine
    from julia_relaxtime_gb300.scan import ScanOptions, gpu_point_solver, read_existing_keys, run_gap_transport_scan

    golden = os.path.join(ROOT, "tests", "golden")
    tmp = tempfile.mkdtemp(prefix="pnjl_scan_")

    def opts(name, xi_values=(0.0, 0.2, 0.4)):
        return ScanOptions(output=os.path.join(tmp, name), xi_values=list(xi_values), tmin_mev=50.0,
                           tmax_mev=300.0, tstep_mev=250.0 / 31.0, mubmin_mev=0.0, mubmax_mev=1200.0,
                           mubstep_mev=1200.0 / 31.0, overwrite=True, resume=False, p_num=64, t_num=8, max_iter=40,
                           boundary_path=os.path.join(golden, "boundary.csv"), cep_path=os.path.join(golden, "cep.csv"))

    eng = GapEngine(p_num=64, t_num=8)
    solver = gpu_point_solver(64, 8, engine=eng)

    def rows_of(path):
        with open(path) as fh:
            lines = [ln.rstrip("\n").split(",") for ln in fh if not ln.startswith("#")]
        head = lines[0]
        return [dict(zip(head, ln)) for ln in lines[1:]]

    for _ in range(args.warmup):
        run_gap_transport_scan(opts("warm.csv"), solver=solver)
    times, launches0 = [], eng.stats()["kernel_launches"]
    for k in range(args.steps):
        t0 = time.perf_counter()
        run_gap_transport_scan(opts(f"gpu{k}.csv"), solver=solver)
        times.append(time.perf_counter() - t0)
    launches = eng.stats()["kernel_launches"] - launches0
    rows = rows_of(os.path.join(tmp, "gpu0.csv"))
    conv = sum(1 for r in rows if r["converged"] == "true")
    line = {"metric": "gap-transport scan rows/s through the drop-in driver (continuation seeds, FP64, ftol 1e-9)",
            "value": conv * args.steps / sum(times), "unit": "rows/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "gap_transport_scan_32x32x3", "rows": len(rows), "p_num": 64, "t_num": 8,
                       "grid": "T 50-300 MeV (32) x mu_B 0-1200 MeV (32) x xi 0, 0.2, 0.4",
                       "seeds": "MultiSeed on each column's first T, PhaseAwareContinuitySeed after it"},
            "gpu_launches": int(launches), "launches_per_scan": launches / args.steps,
            "timing": "host wall clock around run_gap_transport_scan (solves, trackers, K data, CSV)"}
    if not args.no_cpu_baseline:
        # the checker: the same driver over the oracle, all host cores
        from oracle import oracle as orc

        P = orc.default_params()
        nd = orc.Nodes(64, 8)
        threads = os.cpu_count() or 1

        def oracle_solver(T, mu, xi, point_seeds, max_iter):
            o = orc.default_opts(max_iter=max_iter)
            mu3 = np.repeat(np.asarray(mu, dtype=np.float64).reshape(-1, 1), 3, axis=1)
            if point_seeds is None:
                rs = orc.solve_batch(P, nd, T, mu3, xi, multi=True, multiseed_rule=True, opts=o, threads=threads)
            else:
                rs = orc.solve_batch(P, nd, T, mu3, xi, seeds=point_seeds, multi=False, opts=o, threads=threads)
            n = len(rs)
            return {"x": np.array([list(r.x) for r in rs]).reshape(n, 5), "omega": np.array([r.omega for r in rs]),
                    "pressure": np.array([r.pressure for r in rs]), "entropy": np.array([r.entropy for r in rs]),
                    "energy": np.array([r.energy for r in rs]), "rho_norm": np.array([r.rho_norm for r in rs]),
                    "masses": np.array([list(r.masses) for r in rs]).reshape(n, 3),
                    "n_q": np.array([list(r.nq) for r in rs]).reshape(n, 3),
                    "n_aq": np.array([list(r.naq) for r in rs]).reshape(n, 3),
                    "residual_norm": np.array([r.residual_norm for r in rs]),
                    "iterations": np.array([r.iterations for r in rs]), "status": np.array([r.status for r in rs]),
                    "converged": np.array([bool(r.converged) for r in rs])}

        t0 = time.perf_counter()
        run_gap_transport_scan(opts("oracle.csv"), solver=oracle_solver)
        dt = time.perf_counter() - t0
        orows = rows_of(os.path.join(tmp, "oracle.csv"))
        oconv = sum(1 for r in orows if r["converged"] == "true")
        same = sum(1 for a, b in zip(rows, orows)
                   if a["converged"] == b["converged"] and
                   abs(float(a["omega_fm4inv"]) - float(b["omega_fm4inv"])) <= 1e-10 * abs(float(b["omega_fm4inv"])))
        line["cpu_baseline"] = {"value": oconv / dt, "unit": "rows/s", "cores": threads, "kind": "port",
                                "sample": f"the whole scan ({len(orows)} rows) through the same driver"}
        line["rows_agreeing_with_oracle"] = {"rows": len(rows), "same_convergence_and_omega_1e-10": same}
    print(json.dumps(line))
    eng.close()


def run_orders(args):
    """Mixed quadrature orders in one graph launch: the 32 x 32 (T 50-300 MeV, mu 0-400 MeV, xi = 0)
    grid solved with MultiSeed (6 candidates, min-Omega) in mixed precision at p = 64, 128 and 256
    momentum nodes (t = 8), the three segments captured into one CUDA graph (pnjl_plan_*).  Per-point
    errors against the FP64 solve of the same kernel at the same order."""
    import torch

    from julia_relaxtime_gb300.engine import GapEngine, SolveOptions, SolvePlan
    from julia_relaxtime_gb300.pnjl import multiseed_table

    grid = workload_grid("iso_scan_32x32")
    T, mu, _, xi = grid["at"](np.arange(grid["n"]))
    n = T.size
    orders = (64, 128, 256)
    eng = GapEngine(p_num=64, t_num=8)
    dev = torch.device("cuda", 0)
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in (("T", T), ("mu", mu), ("xi", xi))}
    table, hot = multiseed_table(6)
    mixed = SolveOptions(iterations=40, ftol=1e-10, precision="mixed")
    f64 = lambda *sh: torch.empty(*sh, dtype=torch.float64, device=dev)  # noqa: E731
    outs = [{"x": f64(5 * n), "omega": f64(n), "residual_norm": f64(n),
             "converged": torch.empty(n, dtype=torch.uint8, device=dev)} for _ in orders]
    m = d["mu"].data_ptr()
    plan = SolvePlan(eng)
    for p_num, out in zip(orders, outs):
        plan.add(p_num, 8, n, d["T"].data_ptr(), m, m, m, d["xi"].data_ptr(), {k: v.data_ptr() for k, v in out.items()},
                 seed_table=table, seed_table_hot=hot, opts=mixed)
    torch.cuda.synchronize()
    plan.finalize()
    stream = torch.cuda.ExternalStream(eng.stream(), device=dev)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    for _ in range(args.warmup):
        plan.launch()
    eng.synchronize()
    ms, solved = [], 0
    sampler = ClockSampler(0)
    sampler.start()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xFF)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plan.launch()
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
        for out in outs:
            solved += int(((out["converged"] == 1) & (out["residual_norm"] <= 1e-10)).sum().item())
    clocks = sampler.stop()
    st = plan.stats()
    # errors against the FP64 solve of the same kernel at each order
    errs = {}
    for p_num, out in zip(orders, outs):
        eng.set_nodes(p_num, 8)
        ref = eng.solve(T, mu, xi, seed_table=table, seed_table_hot=hot,
                        opts=SolveOptions(iterations=40, ftol=1e-10, precision="fp64"))
        x = out["x"].cpu().numpy().reshape(n, 5)
        om = out["omega"].cpu().numpy()
        conv = out["converged"].cpu().numpy().astype(bool) & ref["converged"]
        same = conv & (np.abs(om - ref["omega"]) <= 1e-10 * np.maximum(np.abs(ref["omega"]), 1.0))
        errs[f"p{p_num}"] = {
            "points": int(conv.sum()), "phase_misassignments": int(np.sum(conv & ~same)),
            "max_abs_dphi": float(np.abs(x[same, :3] - ref["x"][same, :3]).max()),
            "max_rel_dphi": float((np.abs(x[same, :3] - ref["x"][same, :3]) / np.abs(ref["x"][same, :3])).max()),
            "max_abs_dPhi": float(np.abs(x[same, 3:] - ref["x"][same, 3:]).max()),
            "max_rel_domega": float((np.abs(om[same] - ref["omega"][same]) / np.abs(ref["omega"][same])).max())}
    total = sum(ms)
    line = {"metric": METRIC, "value": solved / (total * 1e-3), "unit": "solves/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": "iso_orders_32x32_p64_128_256", "grid": grid["desc"].replace("p64 x t8, ", ""),
                       "segments": "p = 64, 128, 256 x t = 8, one CUDA graph launch per step", "points_per_step":
                       len(orders) * n, "ftol": 1e-10, "max_iter": 40, "precision": "mixed",
                       "l2": "256 MiB device buffer written before every timed step"},
            "gpu_launches": st["kernel_launches"] * args.steps, "clocks": clocks,
            "errors_vs_fp64": errs, "e2e": None}
    print(json.dumps(line))
    plan.close()
    eng.close()


def main():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=("gpu", "reference"))
    ap.add_argument("--workload", default="first_order_2048x2048x9",
                    choices=("first_order_2048x2048x9", "aniso_scan_256x256x9", "surrogate_eval_2p20", "iso_scan_32x32"))
    ap.add_argument("--mode", default="surrogate", choices=("surrogate", "multiseed", "orders", "scan"),
                    help="surrogate: learned seed + mixed precision (headline); multiseed: the MultiSeed table; "
                         "orders: the 32 x 32 isotropic grid at p = 64, 128, 256 in one CUDA graph (mixed "
                         "precision, errors against the FP64 solve of the same kernel); scan: the drop-in "
                         "gap-transport scan driver end to end (32 x 32 x 3, continuation seeds) beside the same "
                         "driver over the oracle")
    ap.add_argument("--precision", default=None, choices=("fp64", "mixed"),
                    help="precision of the timed arm (default: mixed for surrogate, fp64 for multiseed)")
    ap.add_argument("--chunks", type=int, default=None,
                    help="the grid is solved in this many strided slices (default: per workload -- 32, or 2048 "
                         "for the 37.7 M-point first-order scan, 1 for the 32 x 32 grid)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 multi-seed comparison arm")
    ap.add_argument("--cpu-sample", type=int, default=48, help="points per step of the CPU baseline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle check of the arms' roots")
    ap.add_argument("--no-autotune", action="store_true", help="keep the library's default launch shape")
    ap.add_argument("--train-epochs", type=int, default=None, help="training epochs of the network (default 300)")
    ap.add_argument("--train-batch", type=int, default=None, help="training batch (default 1024)")
    ap.add_argument("--train-lr", type=float, default=None, help="peak learning rate (default 4e-3)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    precision = args.precision or ("mixed" if args.mode == "surrogate" else "fp64")

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    grid = workload_grid(args.workload)
    if args.chunks is None:
        args.chunks = grid["chunks"]
    config = {"workload": args.workload, "grid": grid["desc"], "points": int(grid["n"]),
              "points_per_step": int(math.ceil(grid["n"] / world / args.chunks)), "ftol": 1e-10,
              "max_iter": 40, "mode": args.mode, "precision": precision,
              "l2": "256 MiB device buffer written before every timed step"}

    if args.impl == "reference":
        if rank != 0:
            return
        ref = run_reference(args, grid, args.cpu_sample)
        single = single_thread_rate(grid, max(4, args.cpu_sample // 8))
        line = {"metric": METRIC, "value": ref["value"], "unit": "solves/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * ref["seconds"] / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": config, "impl": "reference",
                "cpu_baseline": {"value": ref["value"], "unit": "solves/s", "cores": ref["cores"], "kind": "port",
                                 "sample": ref["sample"], "single_thread": single},
                "e2e": {"value": ref["value"], "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch

    if args.mode == "orders":
        run_orders(args)
        return
    if args.mode == "scan":
        run_scan(args)
        return

    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    torch.cuda.set_device(local_rank)
    from julia_relaxtime_gb300.engine import GapEngine, SolveOptions
    from julia_relaxtime_gb300.learned_seed import default_learned_opts, train_learned_seed
    from julia_relaxtime_gb300.pnjl import DefaultSeed, MultiSeed, multiseed_table

    eng = GapEngine(device=local_rank, p_num=grid["p_num"], t_num=grid["t_num"])
    table, hot = multiseed_table(grid["n_seeds"], grid["extra"])
    train = None
    if args.mode == "surrogate":
        # set-up, untimed: label the 64 x 64 x 5 training grid with the multi-seed solver and
        # train the network on it (both on this GPU); reported as train_s
        tc = grid["train"]
        import dataclasses

        over = {k: v for k, v in (("epochs", args.train_epochs), ("batch", args.train_batch), ("lr", args.train_lr))
                if v is not None}
        tc = dataclasses.replace(tc, **over) if over else tc
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ls = train_learned_seed(eng, tc)
        train = {"seconds": time.perf_counter() - t0,
                 "labels": f"64 x 64 x 5 (T {tc.T_MeV[0]:g}-{tc.T_MeV[1]:g} MeV, mu {tc.mu_MeV[0]:g}-{tc.mu_MeV[1]:g} "
                           f"MeV, xi {tc.xi[0]:g}..{tc.xi[1]:g}) grid, mu_s = {tc.mu_s_ratio:g} mu_u, "
                           f"MultiSeed ({tc.label_seeds + len(tc.label_extra)}) mixed",
                 "epochs": tc.epochs, "batch": tc.batch, "lr": tc.lr}
        arm = Arm("surrogate", eng, table, hot,
                  default_learned_opts(ftol=1e-10, precision=precision, verify_map=ls.verify_map), True)
        train["verify_map_cells_flagged"] = ls.verify_map.fraction()
        train["breakdown"] = ls.timings
        train["verify_map_criteria"] = {"coexisting_phase_within_fm4": tc.map_gap_max, "label_jump_above": tc.map_jump,
                                        "grow_cells": tc.map_grow}
    else:
        arm = Arm("multiseed", eng, table, hot, SolveOptions(iterations=40, ftol=1e-10, precision=precision), False)
    plain = Arm("plain_fp64", eng, table, hot, SolveOptions(iterations=40, ftol=1e-10, precision="fp64"), False)

    # this rank's share of the points: a strided shard (shard_points: no data exchange between
    # ranks), solved in strided slices; slice c holds the shard's points c, c + chunks, ...
    n_local = len(range(rank, grid["n"], world))

    def chunk_points(c):
        return grid["at"](slice_indices(grid["n"], rank, world, args.chunks, c))

    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.ExternalStream(eng.stream(), device=dev)
    maxn = int(math.ceil(n_local / args.chunks))
    d_in = {k: torch.empty(maxn, dtype=torch.float64, device=dev) for k in ("T", "mu", "mu_s", "xi")}
    f64 = lambda *s: torch.empty(*s, dtype=torch.float64, device=dev)  # noqa: E731
    d_out = {"x": f64(maxn * 5), "omega": f64(maxn), "pressure": f64(maxn), "rho_norm": f64(maxn),
             "entropy": f64(maxn), "energy": f64(maxn), "residual_norm": f64(maxn), "masses": f64(maxn * 3),
             "rho": f64(maxn * 3), "n_q": f64(maxn * 3), "n_aq": f64(maxn * 3),
             "iterations": torch.empty(maxn, dtype=torch.int32, device=dev),
             "chosen_seed": torch.empty(maxn, dtype=torch.int32, device=dev),
             "status": torch.empty(maxn, dtype=torch.int32, device=dev),
             "converged": torch.empty(maxn, dtype=torch.uint8, device=dev)}
    ptrs = {k: v.data_ptr() for k, v in d_out.items()}
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)

    def load_chunk(c):
        T, mu_u, mu_s, xi = chunk_points(c)
        n = T.size
        with torch.cuda.stream(stream):
            for k, v in (("T", T), ("mu", mu_u), ("mu_s", mu_s), ("xi", xi)):
                d_in[k][:n].copy_(torch.from_numpy(np.ascontiguousarray(v)))
        stream.synchronize()
        return n

    def run_arm(a: Arm, steps: int, warmup: int, sample_clocks: bool):
        for w in range(warmup):
            n = load_chunk(args.chunks - 1 - (w % args.chunks))
            a.launch(n, d_in, ptrs)
            eng.synchronize()
        sampler = ClockSampler(local_rank) if sample_clocks else None
        rec = {"step_ms": [], "kernel_ms": [], "solved": 0, "flops64": 0.0, "flops32": 0.0, "flops_ff": 0.0,
               "evals": 0, "kinds": {}, "results": [], "k0_ms": [], "k1_ms": [], "k0_flops": [0.0, 0.0, 0.0],
               "k0_evals": 0, "mufu": 0.0, "k0_mufu": 0.0}
        launches0 = eng.stats()["kernel_launches"]
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        if sampler:
            sampler.start()
        for k in range(steps):
            n = load_chunk(k % args.chunks)
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xFF)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            a.launch(n, d_in, ptrs)
            e1.record(stream)
            e1.synchronize()
            rec["step_ms"].append(e0.elapsed_time(e1))
            st = eng.stats()
            rec["kernel_ms"].append(st["last_kernel_ms"])
            rec["evals"] += st["node_evals_fp64"] + st["node_evals_fp32"] + st["node_evals_fp32_thermo"] + \
                st["node_evals_ff"] + st["node_evals_ff_thermo"] + st["node_evals_ff_grad_thermo"]
            f64_, f32_, fff_ = pass_flops(st)
            rec["flops64"] += f64_
            rec["flops32"] += f32_
            rec["flops_ff"] += fff_
            rec["mufu"] += pass_mufu(st)
            # the first kernel alone (the per-point kernel of a learned / per-point solve)
            s0, s1 = eng.stats(kernel=0), eng.stats(kernel=1)
            rec["k0_ms"].append(s0["last_kernel_ms"])
            rec["k1_ms"].append(s1["last_kernel_ms"])
            for j, v in enumerate(pass_flops(s0)):
                rec["k0_flops"][j] += v
            rec["k0_mufu"] += pass_mufu(s0)
            rec["k0_evals"] += s0["node_evals_fp64"] + s0["node_evals_fp32"] + s0["node_evals_fp32_thermo"] + \
                s0["node_evals_ff"] + s0["node_evals_ff_thermo"] + s0["node_evals_ff_grad_thermo"]
            for kk in ("node_evals_fp64_newton", "node_evals_fp64_thermo", "node_evals_fp64_grad",
                       "node_evals_fp64_grad_thermo", "node_evals_fp32", "node_evals_fp32_thermo", "node_evals_ff",
                       "node_evals_ff_thermo", "node_evals_ff_grad_thermo",
                       "seeds_run", "trust_region_runs", "multiseed_fallbacks", "fp64_rescues", "pruned_candidates"):
                rec["kinds"][kk] = rec["kinds"].get(kk, 0) + st[kk]
            conv = d_out["converged"][:n].cpu().numpy().astype(bool)
            res = d_out["residual_norm"][:n].cpu().numpy()
            rec["solved"] += int(np.sum(conv & (res <= 1e-10)))
            rec["results"].append({"converged": conv, "x": d_out["x"][:5 * n].cpu().numpy().reshape(n, 5),
                                   "omega": d_out["omega"][:n].cpu().numpy(), "residual_norm": res, "chunk": k % args.chunks})
        torch.cuda.synchronize()
        rec["clocks"] = sampler.stop() if sampler else None
        rec["launches"] = eng.stats()["kernel_launches"] - launches0
        total_ms = sum(rec["step_ms"])
        solved = rec["solved"]
        if dist is not None:
            t = torch.tensor([total_ms], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            total_ms = float(t.item())
            s_ = torch.tensor([solved], device=dev, dtype=torch.float64)
            dist.all_reduce(s_)
            solved = int(s_.item())
        rec["total_ms"] = total_ms
        rec["value"] = solved / (total_ms * 1e-3)
        return rec

    # launch shape from the library's autotuner on the first slice (untimed set-up)
    tuning = None
    if not args.no_autotune:
        n0 = load_chunk(0)
        m0 = d_in["mu"].data_ptr()
        best, tried = eng.autotune(n0, d_in["T"].data_ptr(), m0, m0, d_in["mu_s"].data_ptr(), d_in["xi"].data_ptr(), ptrs,
                                   seed_table=table, seed_table_hot=hot, opts=arm.opts, learned=arm.learned, reps=2)
        eng.synchronize()
        tuning = {"chosen": best, "candidates": len(tried),
                  "tried": [[t["blocks_per_sm"], t["pipeline_chunks"], t["cert_warps"], round(t["ms"], 3)] for t in tried],
                  "tried_fields": ["blocks_per_sm", "pipeline_chunks", "cert_warps", "ms"]}
    main_rec = run_arm(arm, args.steps, args.warmup, True)

    # the dominant kernel's own launches, for the roofline: the fused kernel (one launch per
    # step) alone between its CUDA events -- the timed run itself when the tuner chose it
    roof_rec = main_rec
    if args.mode == "surrogate" and precision == "mixed" and eng.tuning()["pipeline_chunks"] not in (0, 1):
        tu = eng.tuning()
        eng.set_tuning(32, tu["blocks_per_sm"], pipeline_chunks=1)
        roof_rec = run_arm(arm, args.steps, 0, False)
        eng.set_tuning(32, tu["blocks_per_sm"], pipeline_chunks=tu["pipeline_chunks"])

    # the plain FP64 multi-seed Newton on the same chunks: the denominator of the speed-up and
    # the FP64 judge of the surrogate's phase selection
    plain_line = prec = None
    if args.mode == "surrogate" and not args.no_plain:
        prec = run_arm(plain, args.steps, 1, False)
        mis, dphi, dphi_abs, dPhi, both_n, n_rel = 0, 0.0, 0.0, 0.0, 0, 0
        for r, q in zip(main_rec["results"], prec["results"]):
            both = r["converged"] & q["converged"]
            both_n += int(both.sum())
            om, oq = r["omega"][both], q["omega"][both]
            same = np.abs(om - oq) <= 1e-10 * np.maximum(np.abs(oq), 1.0)
            mis += int(np.sum(~same))
            xr, xq = r["x"][both][same], q["x"][both][same]
            if xr.size:
                d = np.abs(xr[:, :3] - xq[:, :3])
                rel = d / np.maximum(np.abs(xq[:, :3]), 1e-300)
                dphi = max(dphi, float(rel.max()))
                dphi_abs = max(dphi_abs, float(d.max()))
                n_rel += int(np.sum(rel.max(axis=1) > 1e-9))
                dPhi = max(dPhi, float(np.max(np.abs(xr[:, 3:] - xq[:, 3:]))))
        plain_line = {"value": prec["value"], "unit": "solves/s", "ms_per_step": prec["total_ms"] / args.steps,
                      "precision": "fp64", "seeds": seed_count(grid), "speedup": main_rec["value"] / prec["value"],
                      "phase_misassignments": mis, "points_compared": both_n, "max_rel_dphi": dphi,
                      "points_rel_dphi_above_1e-9": n_rel, "max_abs_dphi": dphi_abs, "max_abs_dPhi": dPhi,
                      "work_per_step": {k: v / args.steps for k, v in prec["kinds"].items()}}

    # e2e: the public host-array call (pnjl_solve_batch_learned / pnjl_solve_batch) with pinned
    # host buffers; host<->device copies inside the timed region
    e2e = None
    if not args.no_e2e:
        e2e_solved, e2e_s, h2d, d2h = 0, 0.0, 0, 0
        # the same candidates as the device-array arm (the first n_seeds of MultiSeed)
        e2e_ms = MultiSeed(candidates=MultiSeed().candidates[:grid["n_seeds"]] +
                           [DefaultSeed(tuple(r), tuple(r), "hadron") for r in grid["extra"]])
        for k in range(-1, args.steps):  # k = -1: one untimed call (allocates the pinned staging)
            T_, mu_u, mu_s, xi_ = chunk_points(k)
            n = T_.size
            Th = torch.from_numpy(np.ascontiguousarray(T_)).pin_memory().numpy()
            Mh = torch.from_numpy(np.stack([mu_u, mu_u, mu_s], axis=1)).pin_memory().numpy()
            Xh = torch.from_numpy(np.ascontiguousarray(xi_)).pin_memory().numpy()
            t0 = time.perf_counter()
            if arm.learned:
                r = ls.solve(Th, Mh, Xh, opts=arm.opts, multiseed=e2e_ms)
            else:
                r = eng.solve(Th, Mh, Xh, seed_table=table, seed_table_hot=hot, opts=arm.opts)
            if k < 0:
                continue
            e2e_s += time.perf_counter() - t0
            e2e_solved += int(np.sum(r["converged"] & (r["residual_norm"] <= 1e-10)))
            h2d = 5 * 8 * n  # T, mu_u, mu_d, mu_s, xi
            d2h = sum(v.nbytes for v in r.values())
        e2e = {"value": e2e_solved / e2e_s, "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h)}

    if rank != 0:
        eng.close()
        if dist is not None:
            dist.destroy_process_group()
        return
    peak_fp64 = eng.probe_peak("fp64")
    peak_fp32 = eng.probe_peak("fp32")
    peak_sfu = eng.probe_peak("sfu")
    K = args.steps
    if precision == "fp64":
        kname, k_ms, k_flops, k_evals, k_mufu = "solve_kernel<32>", main_rec["kernel_ms"], \
            [main_rec["flops64"], main_rec["flops32"], main_rec["flops_ff"]], main_rec["evals"], main_rec["mufu"]
    elif args.mode == "surrogate":
        kname, k_ms, k_flops, k_evals, k_mufu = "mixed_fused_kernel<32>", roof_rec["k0_ms"], roof_rec["k0_flops"], \
            roof_rec["k0_evals"], roof_rec["k0_mufu"]
    else:
        kname, k_ms, k_flops, k_evals, k_mufu = "mixed_tasks_kernel<32>", main_rec["kernel_ms"], \
            [main_rec["flops64"], main_rec["flops32"], main_rec["flops_ff"]], main_rec["evals"], main_rec["mufu"]
    avg_k_s = (sum(k_ms) / len(k_ms)) * 1e-3
    ach64 = k_flops[0] / K / avg_k_s
    ach32 = k_flops[1] / K / avg_k_s
    ach_sfu = k_mufu / K / avg_k_s
    step_kernels_ms = sum(roof_rec["kernel_ms"]) / K
    roof = {"bound": "fp64", "kernel": kname, "achieved": ach64 / 1e12, "peak": peak_fp64 / 1e12,
            "unit": "TFLOP/s", "frac": ach64 / peak_fp64,
            "peak_source": "measured in-run (pnjl_probe_peak: FP64 FMA chains on every lane of the GPU); "
                           "no HBM or tensor-core bound applies to this compute-bound path",
            "flop_per_node_flavour": {"newton_pass": FLOP_NEWTON, "thermo_pass": FLOP_THERMO,
                                      "residual_pass": FLOP_GRAD, "residual_thermo_pass": FLOP_GRAD_THERMO,
                                      "newton_pass_fp32": FLOP_NEWTON32, "omega_pass_fp32": FLOP_THERMO32,
                                      "residual_pass_float_float": FLOP_FF, "thermo_pass_float_float": FLOP_FF_THERMO,
                                      "residual_thermo_pass_float_float": FLOP_GRAD_THERMO},
            "node_flavour_evals_per_launch": k_evals / K, "kernel_ms": avg_k_s * 1e3,
            "kernel_share_of_step": avg_k_s * 1e3 / step_kernels_ms if step_kernels_ms > 0 else None,
            "traffic": TRAFFIC.get(kname, {}).get("bytes_per_launch") if args.workload == "aniso_scan_256x256x9"
            else None,
            "traffic_source": TRAFFIC.get(kname, {}).get("source"),
            "fp32": {"achieved": ach32 / 1e12, "peak": peak_fp32 / 1e12, "frac": ach32 / peak_fp32},
            "sfu": {"achieved": ach_sfu / 1e12, "peak": peak_sfu / 1e12, "unit": "Tops/s", "frac": ach_sfu / peak_sfu,
                    "mufu_per_node_flavour": MUFU,
                    "peak_source": "measured in-run (pnjl_probe_peak: ex2.approx chains on every lane)"},
            "float_float_flop_per_launch": k_flops[2] / K}
    launches = main_rec["launches"]
    line = {"metric": METRIC, "value": main_rec["value"], "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": main_rec["total_ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if precision == "fp64" else "f32+f64",
            "data": "synthetic", "config": config, "e2e": e2e, "gpu_launches": int(launches),
            "roofline": roof, "clocks": main_rec["clocks"], "solved": main_rec["solved"], "tuning": tuning,
            "step_ms": {"min": min(main_rec["step_ms"]), "median": statistics.median(main_rec["step_ms"]),
                        "max": max(main_rec["step_ms"])},
            "work_per_step": {k: v / args.steps for k, v in main_rec["kinds"].items()}}
    if train is not None:
        # the whole grid's rate with the set-up (labels, training, verification map) included
        gn = float(grid["n"])
        line["surrogate"] = {"train": train,
                             "amortised": {"value": gn / (gn / main_rec["value"] + train["seconds"]), "unit": "solves/s",
                                           "grid_points": int(gn),
                                           "how": "grid points / (grid points / value + train.seconds)"},
                             "fallback_rate": main_rec["kinds"].get("multiseed_fallbacks", 0) /
                             max(1, config["points_per_step"] * args.steps),
                             "verify": {"seeds": seed_count(grid) if arm.opts.verify_seeds < 0 else arm.opts.verify_seeds,
                                        "region": "verification map (flagged cells of the label grid)"
                                        if arm.opts.verify_map is not None else
                                        f"T < {arm.opts.verify_T_max_MeV} MeV",
                                        "max_step": arm.opts.verify_max_step}}
    if plain_line is not None:
        line["plain_fp64"] = plain_line
    if not args.no_cpu_baseline:
        class A:  # noqa: N801
            warmup, steps = 0, 1
        ref = run_reference(A, grid, args.cpu_sample)
        line["cpu_baseline"] = {"value": ref["value"], "unit": "solves/s", "cores": ref["cores"], "kind": "port",
                                "sample": ref["sample"],
                                "single_thread": single_thread_rate(grid, max(4, args.cpu_sample // 8))}
        if prec is not None and not args.no_parity:
            # the checker: both timed arms' roots against the oracle's
            line["parity"] = parity_vs_oracle(grid, {"surrogate_mixed": main_rec["results"],
                                                     "plain_fp64": prec["results"]}, chunk_points)
    print(json.dumps(line))
    eng.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
