"""Batched gap-equation scan with the CSV of scripts/relaxtime/run_gap_transport_scan.jl.

The reference walks xi -> muB -> T one point at a time (run_gap_transport_scan.jl:407-417):
the first T of each (xi, muB) column is solved with MultiSeed, every later T with a
PhaseAwareContinuitySeed tracker of that column (:412-441).  Columns are independent, so here
all columns of one xi advance together: step k solves the k-th temperature of every column
in one GPU launch (first points in MultiSeed mode, the others with their tracker's seed and
the MultiSeed fallback), then each tracker is updated exactly as the reference updates it.
Rows are written in the reference's order with the same 47 columns, metadata lines and
resume keys (scripts/utils/scan_csv.jl:18-90).  The tau / transport columns belong to the
relaxation-time chain, which this engine does not compute; they are written as NaN.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from typing import Callable, Sequence

import numpy as np

from . import _capi as api
from .constants import HBARC_MEV_FM
from .pnjl import PhaseAwareContinuitySeed, FixedMu, MultiSeed

HEADER = [
    "T_MeV", "muq_MeV", "muB_MeV", "xi",
    "T_fm", "muq_fm",
    "converged", "iterations", "residual_norm",
    "Phi", "Phibar",
    "m_u", "m_d", "m_s",
    "rho_baryon", "rho_norm",
    "omega_fm4inv", "P_fm4inv", "epsilon_fm4inv", "s_fm3inv",
    "omega_MeV_fm3", "P_MeV_fm3", "epsilon_MeV_fm3",
    "eps_minus_3P_over_T4",
    "n_u", "n_d", "n_s", "n_ubar", "n_dbar", "n_sbar",
    "tau_u", "tau_d", "tau_s", "tau_ubar", "tau_dbar", "tau_sbar",
    "tauinv_u", "tauinv_d", "tauinv_s", "tauinv_ubar", "tauinv_dbar", "tauinv_sbar",
    "eta", "sigma", "zeta", "eta_over_s", "zeta_over_s",
]


def julia_string(x: float) -> str:
    """Julia's string(::Float64): shortest round-trip digits; plain notation for decimal
    exponents -4..5 ("120.0", "0.0001"), else "d.ddde-5" / "1.0e6" (no '+', no padding)."""
    x = float(x)
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "Inf" if x > 0 else "-Inf"
    if x == 0.0:
        return "-0.0" if math.copysign(1.0, x) < 0 else "0.0"
    r = repr(x)
    sign = "-" if r.startswith("-") else ""
    r = r.lstrip("-")
    if "e" in r:
        mant, ex = r.split("e")
        exp10 = int(ex)
    else:
        mant, exp10 = r, 0
    if "." in mant:
        ip, fp = mant.split(".")
    else:
        ip, fp = mant, ""
    digits = (ip + fp).lstrip("0")
    # decimal exponent of the leading digit
    if ip.strip("0"):
        lead = len(ip.lstrip("0")) - 1 + exp10
    else:
        lead = -(len(fp) - len(fp.lstrip("0")) + 1) + exp10
    digits = digits.rstrip("0") or "0"
    if -4 <= lead <= 5:
        if lead >= 0:
            if len(digits) <= lead + 1:
                s = digits + "0" * (lead + 1 - len(digits)) + ".0"
            else:
                s = digits[: lead + 1] + "." + digits[lead + 1:]
        else:
            s = "0." + "0" * (-lead - 1) + digits
        return sign + s
    m = digits[0] + "." + (digits[1:] if len(digits) > 1 else "0")
    return f"{sign}{m}e{lead}"


@dataclass
class ScanOptions:
    """CLI options of run_gap_transport_scan.jl:97-237 that concern the gap solve."""
    output: str = os.path.join("data", "outputs", "results", "relaxtime", "gap_transport_scan.csv")
    xi_values: Sequence[float] = (0.0,)
    tmin_mev: float = 50.0
    tmax_mev: float = 200.0
    tstep_mev: float = 10.0
    mubmin_mev: float = 0.0
    mubmax_mev: float = 1200.0
    mubstep_mev: float = 60.0
    overwrite: bool = False
    resume: bool = True
    p_num: int = 12
    t_num: int = 6
    max_iter: int = 40
    boundary_path: str | None = None
    cep_path: str | None = None
    precision: str = "fp64"
    metadata: dict = field(default_factory=dict)


def julia_range(start: float, stop: float, step: float) -> list[float]:
    """collect(range(start; stop, step)) for the grids of the scan (start + k*step)."""
    n = int(math.floor((stop - start) / step + 1e-10)) + 1
    return [float(start) + k * float(step) for k in range(max(n, 0))]


# A point solver takes (T_fm[n], mu_fm[n], xi[n], point_seeds[n,5] or None, max_iter) and
# returns the per-point result arrays (the keys of engine.BatchResult).
PointSolver = Callable[..., dict]


def gpu_point_solver(p_num: int, t_num: int, precision: str = "fp64", engine=None) -> PointSolver:
    from .pnjl import solve_batch

    def solver(T, mu, xi, point_seeds, max_iter):
        return solve_batch(T, mu, xi, seed_strategy=None if point_seeds is not None else MultiSeed(),
                           point_seeds=point_seeds, p_num=p_num, t_num=t_num, iterations=max_iter,
                           precision=precision, engine=engine)

    return solver


def scan_rows(opts: ScanOptions, solver: PointSolver, skip: set | None = None) -> list[dict]:
    """Solve the scan grid and return one dict per row, in the reference's order."""
    T_values = julia_range(opts.tmin_mev, opts.tmax_mev, opts.tstep_mev)
    muB_values = sorted(set(float(v) for v in julia_range(opts.mubmin_mev, opts.mubmax_mev, opts.mubstep_mev)))
    skip = skip or set()
    rows = []
    for xi in opts.xi_values:
        xi = float(xi)
        trackers = [PhaseAwareContinuitySeed(xi, boundary_path=opts.boundary_path, cep_path=opts.cep_path)
                    for _ in muB_values]
        col_rows: list[list] = [[None] * len(T_values) for _ in muB_values]
        for k, T_mev in enumerate(T_values):
            T_fm = T_mev / HBARC_MEV_FM
            first, cont = [], []
            for c, muB in enumerate(muB_values):
                if (T_mev, muB, xi) in skip:
                    continue
                (first if trackers[c].previous_solution is None else cont).append(c)
            for group, per_point in ((first, False), (cont, True)):
                if not group:
                    continue
                mus = np.array([muB_values[c] / 3.0 / HBARC_MEV_FM for c in group])
                Ts = np.full(len(group), T_fm)
                xis = np.full(len(group), xi)
                seeds = None
                if per_point:
                    seeds = np.array([trackers[c].get_seed([T_fm, mus[j]], FixedMu()) for j, c in enumerate(group)])
                res = solver(Ts, mus, xis, seeds, opts.max_iter)
                for j, c in enumerate(group):
                    if int(res["status"][j]) in (api.PNJL_POINT_EXCEPTION, api.PNJL_POINT_ALL_SEEDS_FAILED):
                        # the reference raises here; the scan records the point as not converged
                        pass
                    muq_mev = muB_values[c] / 3.0
                    conv = bool(res["converged"][j])
                    if conv:
                        trackers[c].update(res["x"][j], T_mev, muq_mev)
                    col_rows[c][k] = _row(T_mev, muq_mev, muB_values[c], xi, T_fm, mus[j], res, j)
        for c in range(len(muB_values)):
            for k in range(len(T_values)):
                if col_rows[c][k] is not None:
                    rows.append(col_rows[c][k])
    return rows


def _row(T_mev, muq_mev, muB_mev, xi, T_fm, muq_fm, res, j) -> dict:
    x = res["x"][j]
    nq, naq = res["n_q"][j], res["n_aq"][j]
    rho_baryon = ((nq[0] - naq[0]) + (nq[1] - naq[1]) + (nq[2] - naq[2])) / 3.0
    omega, P, eps, s = float(res["omega"][j]), float(res["pressure"][j]), float(res["energy"][j]), float(res["entropy"][j])
    e3p = (eps - 3.0 * P) / T_fm ** 4 if (math.isfinite(eps) and math.isfinite(P) and T_fm != 0.0) else float("nan")
    nan = float("nan")
    return {
        "T_MeV": T_mev, "muq_MeV": muq_mev, "muB_MeV": muB_mev, "xi": xi, "T_fm": T_fm, "muq_fm": muq_fm,
        "converged": bool(res["converged"][j]), "iterations": int(res["iterations"][j]),
        "residual_norm": float(res["residual_norm"][j]), "Phi": float(x[3]), "Phibar": float(x[4]),
        "m_u": float(res["masses"][j][0]), "m_d": float(res["masses"][j][1]), "m_s": float(res["masses"][j][2]),
        "rho_baryon": rho_baryon, "rho_norm": rho_baryon / 0.16,
        "omega_fm4inv": omega, "P_fm4inv": P, "epsilon_fm4inv": eps, "s_fm3inv": s,
        "omega_MeV_fm3": omega * HBARC_MEV_FM, "P_MeV_fm3": P * HBARC_MEV_FM, "epsilon_MeV_fm3": eps * HBARC_MEV_FM,
        "eps_minus_3P_over_T4": e3p,
        "n_u": float(nq[0]), "n_d": float(nq[1]), "n_s": float(nq[2]),
        "n_ubar": float(naq[0]), "n_dbar": float(naq[1]), "n_sbar": float(naq[2]),
        **{k: nan for k in HEADER[30:]},
        "status": int(res["status"][j]), "phi": np.array(x[:3]),
    }


def format_row(r: dict) -> str:
    out = []
    for k in HEADER:
        v = r[k]
        if isinstance(v, bool):
            out.append("true" if v else "false")
        elif isinstance(v, (int, np.integer)):
            out.append(str(int(v)))
        else:
            out.append(julia_string(v))
    return ",".join(out)


def read_existing_keys(path: str, key_cols=("T_MeV", "muB_MeV", "xi")) -> set:
    """scripts/utils/scan_csv.jl:53-90."""
    keys: set = set()
    if not os.path.isfile(path):
        return keys
    with open(path) as fh:
        header = None
        for line in fh:
            s = line.strip()
            if not s or s.startswith("#"):
                continue
            if header is None:
                header = [c.strip() for c in s.split(",")]
                if any(c not in header for c in key_cols):
                    return keys
                idx = [header.index(c) for c in key_cols]
                continue
            parts = s.split(",")
            if len(parts) < max(idx) + 1:
                continue
            try:
                keys.add(tuple(float(parts[i].strip()) for i in idx))
            except ValueError:
                continue
    return keys


def run_gap_transport_scan(opts: ScanOptions, solver: PointSolver | None = None) -> str:
    """The gap part of run_scan (run_gap_transport_scan.jl:362-550), writing opts.output."""
    solver = solver or gpu_point_solver(opts.p_num, opts.t_num, opts.precision)
    d = os.path.dirname(opts.output)
    if d:
        os.makedirs(d, exist_ok=True)
    existing = read_existing_keys(opts.output) if (opts.resume and os.path.isfile(opts.output) and not opts.overwrite) else set()
    if opts.overwrite and os.path.isfile(opts.output):
        os.remove(opts.output)
    new_file = not os.path.isfile(opts.output) or os.path.getsize(opts.output) == 0
    rows = scan_rows(opts, solver, skip=existing)
    with open(opts.output, "a") as fh:
        if new_file:
            meta = {"schema": "scan_csv_v1", "title": "gap_transport_scan",
                    "script": "scripts/relaxtime/run_gap_transport_scan.jl", "engine": "libpnjl_cuda",
                    "p_num": str(opts.p_num), "t_num": str(opts.t_num), "precision": opts.precision}
            meta.update(opts.metadata)
            for k, v in meta.items():
                fh.write(f"# {k}: {v}\n")
            fh.write(",".join(HEADER) + "\n")
        for r in rows:
            fh.write(format_row(r) + "\n")
        fh.flush()
    return opts.output


def main(argv: Sequence[str] | None = None):
    """CLI with the reference's flag names (run_gap_transport_scan.jl:97-237, gap part)."""
    import argparse

    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--output", default=ScanOptions.output)
    ap.add_argument("--xi", default="0.0", help="comma-separated xi values")
    ap.add_argument("--tmin", type=float, default=50.0)
    ap.add_argument("--tmax", type=float, default=200.0)
    ap.add_argument("--tstep", type=float, default=10.0)
    ap.add_argument("--mubmin", type=float, default=0.0)
    ap.add_argument("--mubmax", type=float, default=1200.0)
    ap.add_argument("--mubstep", type=float, default=60.0)
    ap.add_argument("--overwrite", action="store_true")
    ap.add_argument("--no-resume", action="store_true")
    ap.add_argument("--p-num", type=int, default=12)
    ap.add_argument("--t-num", type=int, default=6)
    ap.add_argument("--max-iter", type=int, default=40)
    ap.add_argument("--boundary", default=None, help="boundary.csv of the phase-aware seed")
    ap.add_argument("--cep", default=None, help="cep.csv of the phase-aware seed")
    ap.add_argument("--precision", default="fp64", choices=("fp64", "mixed"))
    a = ap.parse_args(argv)
    opts = ScanOptions(output=a.output, xi_values=[float(v) for v in a.xi.split(",")], tmin_mev=a.tmin,
                       tmax_mev=a.tmax, tstep_mev=a.tstep, mubmin_mev=a.mubmin, mubmax_mev=a.mubmax,
                       mubstep_mev=a.mubstep, overwrite=a.overwrite, resume=not a.no_resume, p_num=a.p_num,
                       t_num=a.t_num, max_iter=a.max_iter, boundary_path=a.boundary, cep_path=a.cep,
                       precision=a.precision)
    print(run_gap_transport_scan(opts))


if __name__ == "__main__":
    main()
