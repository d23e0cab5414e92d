"""Adapters that let host-side drivers of the package run on the CPU oracle in tests.

The scan driver (julia_relaxtime_gb300.scan) takes a point solver; the GPU one is the
product path.  These oracle-backed solvers exist only so that the host logic (trackers,
ordering, CSV) can be checked without a GPU.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402

GOLDEN = os.path.join(ROOT, "tests", "golden")


def results_to_arrays(rs) -> dict:
    n = len(rs)
    out = {
        "x": np.array([list(r.x) for r in rs]).reshape(n, 5),
        "omega": np.array([r.omega for r in rs]),
        "pressure": np.array([r.pressure for r in rs]),
        "rho_norm": np.array([r.rho_norm for r in rs]),
        "entropy": np.array([r.entropy for r in rs]),
        "energy": np.array([r.energy for r in rs]),
        "masses": np.array([list(r.masses) for r in rs]).reshape(n, 3),
        "rho": np.array([list(r.rho) for r in rs]).reshape(n, 3),
        "n_q": np.array([list(r.nq) for r in rs]).reshape(n, 3),
        "n_aq": np.array([list(r.naq) for r in rs]).reshape(n, 3),
        "residual_norm": np.array([r.residual_norm for r in rs]),
        "iterations": np.array([r.iterations for r in rs], dtype=np.int32),
        "chosen_seed": np.array([r.chosen_seed for r in rs], dtype=np.int32),
        "status": np.array([r.status for r in rs], dtype=np.int32),
        "converged": np.array([bool(r.converged) for r in rs]),
    }
    return out


def oracle_point_solver(p_num: int, t_num: int, threads: int = 0, **optkw):
    P = orc.default_params()
    nd = orc.Nodes(p_num, t_num)

    def solver(T, mu, xi, point_seeds, max_iter):
        opts = orc.default_opts(max_iter=max_iter, **optkw)
        mu3 = np.repeat(np.asarray(mu, dtype=np.float64).reshape(-1, 1), 3, axis=1)
        if point_seeds is None:
            rs = orc.solve_batch(P, nd, T, mu3, xi, multi=True, multiseed_rule=True, opts=opts, threads=threads)
        else:
            rs = orc.solve_batch(P, nd, T, mu3, xi, seeds=point_seeds, multi=False, opts=opts, threads=threads)
        return results_to_arrays(rs)

    return solver


def read_csv(path):
    import csv

    with open(os.path.join(GOLDEN, path) if not os.path.isabs(path) else path) as fh:
        rows = [r for r in csv.DictReader(line for line in fh if not line.startswith("#"))]
    return rows
