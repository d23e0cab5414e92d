"""Batched gap-equation scan with the CSV of scripts/relaxtime/run_gap_transport_scan.jl.

The reference walks xi -> muB -> T one point at a time (run_gap_transport_scan.jl:407-417):
the first T of each (xi, muB) column is solved with MultiSeed, every later T with a
PhaseAwareContinuitySeed tracker of that column (:412-441).  Columns are independent, so here
the columns of every xi advance together: step k solves the k-th temperature of every column
in at most two GPU launches (first points in MultiSeed mode, the others with their tracker's
seed and the MultiSeed fallback), then each tracker is updated exactly as the reference
updates it.
Rows are written in the reference's order with the same 47 columns, metadata lines and
resume keys (scripts/utils/scan_csv.jl:18-90).  Each row also keeps the point's K data
(build_K_data, :297-305: the one-loop A per flavour, G^f and the effective couplings, from
the GPU) -- the relaxation-time chain's input; the tau / transport columns themselves belong
to that chain, which this engine does not compute, and are written as NaN.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from typing import Callable, Sequence

import numpy as np

from . import _capi as api
from .constants import HBARC_MEV_FM, PNJLParams
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
    exponents -4..5 ("120.0", "0.0001"), else "d.ddde-5" / "1.0e6" (no '+', no padding).
    For 1e-4 <= |x| < 1e6 that is Python's repr (the same shortest digits, plain notation)."""
    x = float(x)
    if x != x:
        return "NaN"
    if 1e-4 <= abs(x) < 1e6:
        return repr(x)
    return _julia_string_general(x)


def _julia_string_general(x: float) -> str:
    """julia_string for every double, from the digits of repr."""
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
    # the PNJL parameter profile (Constants_PNJL.jl:82-103); None = the built-in default.
    # rho_norm divides by its rho0 (run_gap_transport_scan.jl:500)
    params: PNJLParams | None = None


def julia_range(start: float, stop: float, step: float) -> list[float]:
    """collect(range(start; stop, step)) for the grids of the scan (start + k*step)."""
    n = int(math.floor((stop - start) / step + 1e-10)) + 1
    return [float(start) + k * float(step) for k in range(max(n, 0))]


# A point solver takes (T_fm[n], mu_fm[n], xi[n], point_seeds[n,5] or None, max_iter) and
# returns the per-point result arrays (the keys of engine.BatchResult).
PointSolver = Callable[..., dict]


def gpu_point_solver(p_num: int, t_num: int, precision: str = "fp64", engine=None,
                     params: PNJLParams | None = None, kdata: bool = True) -> PointSolver:
    """The GPU point solver of the scan; with kdata, each result also carries build_K_data
    (run_gap_transport_scan.jl:297-305, computed for every point as the script does) under
    "kdata": {field: [n]}."""
    from .pnjl import default_engine, solve_batch

    eng = engine or default_engine(p_num, t_num, params=params)

    def solver(T, mu, xi, point_seeds, max_iter):
        res = solve_batch(T, mu, xi, seed_strategy=None if point_seeds is not None else MultiSeed(),
                          point_seeds=point_seeds, p_num=p_num, t_num=t_num, iterations=max_iter,
                          precision=precision, engine=eng)
        if kdata:
            res["kdata"] = eng.kdata(T, mu, mu, res["masses"], res["x"])
        return res

    return solver


def scan_rows(opts: ScanOptions, solver: PointSolver, skip: set | None = None) -> list[dict]:
    """Solve the scan grid and return one dict per row, in the reference's order.

    The reference walks xi -> muB -> T (run_gap_transport_scan.jl:407-417) with one
    continuation tracker per (xi, muB) column.  Columns are independent, so one temperature
    of every column of every xi is solved together: at most two launches per temperature,
    one for the columns' first points (MultiSeed) and one for the continued columns (each
    tracker's seed, MultiSeed fallback)."""
    T_values = julia_range(opts.tmin_mev, opts.tmax_mev, opts.tstep_mev)
    muB_values = sorted(set(float(v) for v in julia_range(opts.mubmin_mev, opts.mubmax_mev, opts.mubstep_mev)))
    rho0 = (opts.params or PNJLParams.default()).rho0
    skip = skip or set()
    xis = [float(x) for x in opts.xi_values]
    cols = [(ix, c) for ix in range(len(xis)) for c in range(len(muB_values))]
    trackers = {col: PhaseAwareContinuitySeed(xis[col[0]], boundary_path=opts.boundary_path,
                                              cep_path=opts.cep_path) for col in cols}
    col_rows = {col: [None] * len(T_values) for col in cols}
    for k, T_mev in enumerate(T_values):
        T_fm = T_mev / HBARC_MEV_FM
        first, cont = [], []
        for col in cols:
            if (T_mev, muB_values[col[1]], xis[col[0]]) in skip:
                continue
            (first if trackers[col].previous_solution is None else cont).append(col)
        for group, per_point in ((first, False), (cont, True)):
            if not group:
                continue
            mus = np.array([muB_values[c] / 3.0 / HBARC_MEV_FM for _, c in group])
            Ts = np.full(len(group), T_fm)
            xa = np.array([xis[ix] for ix, _ in group])
            seeds = None
            if per_point:
                seeds = np.array([trackers[col].get_seed([T_fm, mus[j]], FixedMu()) for j, col in enumerate(group)])
            res = solver(Ts, mus, xa, seeds, opts.max_iter)
            for j, col in enumerate(group):
                # a point whose seeds all failed (the reference raises there) is written as
                # not converged
                ix, c = col
                muq_mev = muB_values[c] / 3.0
                if bool(res["converged"][j]):
                    trackers[col].update(res["x"][j], T_mev, muq_mev)
                col_rows[col][k] = _row(T_mev, muq_mev, muB_values[c], xis[ix], T_fm, mus[j], res, j, rho0)
    rows = []
    for col in cols:
        rows.extend(r for r in col_rows[col] if r is not None)
    return rows


def _row(T_mev, muq_mev, muB_mev, xi, T_fm, muq_fm, res, j, rho0: float) -> dict:
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
        "rho_baryon": rho_baryon, "rho_norm": rho_baryon / rho0,
        "omega_fm4inv": omega, "P_fm4inv": P, "epsilon_fm4inv": eps, "s_fm3inv": s,
        "omega_MeV_fm3": omega * HBARC_MEV_FM, "P_MeV_fm3": P * HBARC_MEV_FM, "epsilon_MeV_fm3": eps * HBARC_MEV_FM,
        "eps_minus_3P_over_T4": e3p,
        "n_u": float(nq[0]), "n_d": float(nq[1]), "n_s": float(nq[2]),
        "n_ubar": float(naq[0]), "n_dbar": float(naq[1]), "n_sbar": float(naq[2]),
        **{k: nan for k in HEADER[30:]},
        "status": int(res["status"][j]), "phi": np.array(x[:3]),
        # build_K_data of the point (the relaxation-time chain's input), when the solver gives it
        "kdata": {k: float(v[j]) for k, v in res["kdata"].items()} if "kdata" in res else None,
    }


def format_row(r: dict) -> str:
    out = []
    for k in HEADER:
        v = r[k]
        if type(v) is float:  # most columns
            out.append(julia_string(v))
        elif isinstance(v, bool):
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
    solver = solver or gpu_point_solver(opts.p_num, opts.t_num, opts.precision, params=opts.params)
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
    ap.add_argument("--profile", default=None, help="PNJL parameter profile (default: $PNJL_PARAM_PROFILE)")
    ap.add_argument("--config-dir", default=None, help="directory of the profile .toml files")
    a = ap.parse_args(argv)
    params = PNJLParams.load(a.profile, a.config_dir) if (a.profile or a.config_dir) else None
    opts = ScanOptions(output=a.output, xi_values=[float(v) for v in a.xi.split(",")], tmin_mev=a.tmin,
                       tmax_mev=a.tmax, tstep_mev=a.tstep, mubmin_mev=a.mubmin, mubmax_mev=a.mubmax,
                       mubstep_mev=a.mubstep, overwrite=a.overwrite, resume=not a.no_resume, p_num=a.p_num,
                       t_num=a.t_num, max_iter=a.max_iter, boundary_path=a.boundary, cep_path=a.cep,
                       precision=a.precision, params=params)
    print(run_gap_transport_scan(opts))


if __name__ == "__main__":
    main()


# ---------------------------------------------------------------------------------------
# TmuScan (src/pnjl/scans/TmuScan.jl): T-mu scan with phase-aware continuation along mu.

TMU_HEADER = ["T_MeV", "mu_MeV", "xi", "pressure_fm4", "rho", "entropy_fm3", "energy_fm4", "phi_u", "phi_d",
              "phi_s", "Phi1", "Phi2", "M_u_MeV", "M_d_MeV", "M_s_MeV", "iterations", "residual_norm", "converged",
              "message"]  # TmuScan.jl:62-82
TMU_ACCEPTABLE_RESIDUAL = 1e-4  # TmuScan.jl:60


def _fmt6(x) -> str:
    """@sprintf("%.6f", x) as Julia prints it (NaN, Inf, -Inf spelled as Julia does)."""
    x = float(x)
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "Inf" if x > 0 else "-Inf"
    return "%.6f" % x


def _tmu_key(T, mu, xi):
    return (round(float(T), 6), round(float(mu), 6), round(float(xi), 6))


def _tmu_load_completed(path: str) -> set:
    """TmuScan.jl:243-264: keys of the rows already in the file."""
    done: set = set()
    if not os.path.isfile(path):
        return done
    with open(path) as fh:
        next(fh, None)
        for line in fh:
            cols = line.strip().split(",")
            if len(cols) < 3:
                continue
            try:
                done.add(_tmu_key(float(cols[0]), float(cols[1]), float(cols[2])))
            except ValueError:
                continue
    return done


def _tmu_success(r) -> bool:
    """TmuScan.jl:428-436: converged, or a finite residual <= 1e-4."""
    if r is None:
        return False
    return bool(r["converged"]) or (math.isfinite(r["residual_norm"]) and r["residual_norm"] <= TMU_ACCEPTABLE_RESIDUAL)


def _tmu_failure(label: str, msg: str, r) -> str:
    """TmuScan.jl:521-534."""
    base = f"seed[{label}] failed"
    if r is not None:
        base += f" (iterations={r['iterations']}, residual={_fmt6(r['residual_norm'])}, converged=false)"
    return base if not msg else f"{base}: {msg}"


def _tmu_pick(res, j) -> dict | None:
    """One point of a batch result as the fields TmuScan reads; None where the reference's
    solve raised (its _solve_point catches the exception, TmuScan.jl:380-400)."""
    if int(res["status"][j]) == api.PNJL_POINT_EXCEPTION:
        return None
    return {"x": np.array(res["x"][j], dtype=np.float64), "converged": bool(res["converged"][j]),
            "residual_norm": float(res["residual_norm"][j]), "iterations": int(res["iterations"][j]),
            "pressure": float(res["pressure"][j]), "rho_norm": float(res["rho_norm"][j]),
            "entropy": float(res["entropy"][j]), "energy": float(res["energy"][j]),
            "masses": np.array(res["masses"][j], dtype=np.float64)}


def _tmu_seed_candidates(tracker, cache: dict, T, mu, xi, T_fm, mu_fm):
    """_build_seed_candidates_v2 (TmuScan.jl:267-301)."""
    from .pnjl import HADRON_SEED_5, QUARK_SEED_5

    cands = []
    if tracker is not None:
        label = "phase_aware_default" if tracker.previous_solution is None else "phase_aware_continuity"
        cands.append((label, np.array(tracker.get_seed([T_fm, mu_fm], FixedMu()), dtype=np.float64)))
    key = (round(float(T), 6), round(float(xi), 6))
    if key in cache:
        cands.append(("continuation", cache[key].copy()))
    quark, hadron = ("quark", np.array(QUARK_SEED_5)), ("hadron", np.array(HADRON_SEED_5))
    cands.extend([quark, hadron] if (T > 150 or mu > 300) else [hadron, quark])
    return cands


def tmu_scan_rows(T_values, mu_values, xi_values, solver: PointSolver, *, use_phase_aware: bool = True,
                  max_iter: int = 1000, boundary_path: str | None = None, cep_path: str | None = None,
                  skip: set | None = None):
    """The scan of run_tmu_scan (TmuScan.jl:120-234) as batched solves: every (xi, T) row walks mu
    with its own tracker (the reference resets one tracker per T), so all rows advance together --
    step k solves the k-th mu of every row, trying the rows' k-th seed candidates in one launch per
    candidate rank.  Returns the rows in the reference's order (xi, T, mu) and the statistics."""
    skip = skip or set()
    rows_idx = [(float(xi), float(T)) for xi in xi_values for T in T_values]
    trackers = {}
    for xi, T in rows_idx:
        if not use_phase_aware:
            trackers[(xi, T)] = None
            continue
        try:
            trackers[(xi, T)] = PhaseAwareContinuitySeed(xi, boundary_path=boundary_path, cep_path=cep_path)
        except (OSError, ValueError, KeyError):
            trackers[(xi, T)] = PhaseAwareContinuitySeed()  # no boundary data: plain continuation
    cache: dict = {}
    out = {key: [None] * len(mu_values) for key in rows_idx}
    stats = {"total": 0, "success": 0, "failure": 0, "skipped": 0}
    for m, mu in enumerate(mu_values):
        mu = float(mu)
        active = []
        for key in rows_idx:
            stats["total"] += 1
            if _tmu_key(key[1], mu, key[0]) in skip:
                stats["skipped"] += 1
                continue
            active.append(key)
        if not active:
            continue
        cands = {}
        for xi, T in active:
            cands[(xi, T)] = _tmu_seed_candidates(trackers[(xi, T)], cache, T, mu, xi, T / HBARC_MEV_FM,
                                                  mu / HBARC_MEV_FM)
        msgs = {key: [] for key in active}
        final = {}
        pending = list(active)
        rank = 0
        while pending:
            batch = [key for key in pending if rank < len(cands[key])]
            for key in pending:
                if rank >= len(cands[key]):
                    final[key] = (None, " | ".join(x for x in msgs[key] if x))
            if not batch:
                break
            T_arr = np.array([k[1] / HBARC_MEV_FM for k in batch])
            res = solver(T_arr, np.full(len(batch), mu / HBARC_MEV_FM), np.array([k[0] for k in batch]),
                         np.array([cands[k][rank][1] for k in batch]), max_iter)
            nxt = []
            for j, key in enumerate(batch):
                r = _tmu_pick(res, j)
                msg = "" if r is not None else "solver exception"
                if _tmu_success(r):
                    final[key] = (r, msg)
                else:
                    msgs[key].append(_tmu_failure(cands[key][rank][0], msg, r))
                    nxt.append(key)
            pending = nxt
            rank += 1
        # _refine_result (TmuScan.jl:406-425): near-converged successes are solved again from
        # their own solution
        near = [k for k, (r, _) in final.items() if r is not None and not r["converged"]]
        refine_msg = {}
        if near:
            res = solver(np.array([k[1] / HBARC_MEV_FM for k in near]), np.full(len(near), mu / HBARC_MEV_FM),
                         np.array([k[0] for k in near]), np.array([final[k][0]["x"] for k in near]), max_iter)
            for j, key in enumerate(near):
                r2 = _tmu_pick(res, j)
                if r2 is not None and r2["converged"]:
                    final[key] = (r2, final[key][1])
                    refine_msg[key] = "refined from near-converged seed"
                else:
                    refine_msg[key] = "" if r2 is not None else "solver exception"
        for key in active:
            r, msg = final[key]
            parts = list(msgs[key])
            if r is not None:
                promote = ""
                if not r["converged"]:  # _promote_success (TmuScan.jl:439-468)
                    r = dict(r, converged=True)
                    promote = f"force-marked converged (residual {_fmt6(r['residual_norm'])})"
                parts += [msg, promote, refine_msg.get(key, "")]
                xi, T = key
                if trackers[key] is not None:
                    trackers[key].update(r["x"], T, mu)
                cache[(round(T, 6), round(xi, 6))] = r["x"].copy()
                stats["success"] += 1
            else:
                parts = [msg] if msg else parts
                stats["failure"] += 1
            out[key][m] = (key[1], mu, key[0], r, " | ".join(p for p in parts if p))
    rows = [out[key][m] for key in rows_idx for m in range(len(mu_values)) if out[key][m] is not None]
    return rows, stats


def format_tmu_row(T, mu, xi, r, message: str) -> str:
    """_write_row (TmuScan.jl:471-515)."""
    q = f'"{message}"' if message else ""
    if r is None:
        vals = [_fmt6(T), _fmt6(mu), _fmt6(xi)] + ["NaN"] * 12 + ["-1", "NaN", "false", q]
        return ",".join(vals)
    x, M = r["x"], r["masses"] * HBARC_MEV_FM
    vals = [_fmt6(T), _fmt6(mu), _fmt6(xi), _fmt6(r["pressure"]), _fmt6(r["rho_norm"]), _fmt6(r["entropy"]),
            _fmt6(r["energy"]), _fmt6(x[0]), _fmt6(x[1]), _fmt6(x[2]), _fmt6(x[3]), _fmt6(x[4]),
            _fmt6(M[0]), _fmt6(M[1]), _fmt6(M[2]), str(int(r["iterations"])), _fmt6(r["residual_norm"]),
            "true" if r["converged"] else "false", q]
    return ",".join(vals)


def run_tmu_scan(*, T_values=None, mu_values=None, xi_values=(0.0,),
                 output_path: str = os.path.join("data", "outputs", "results", "pnjl", "tmu_scan.csv"),
                 overwrite: bool = False, resume: bool = True, use_phase_aware: bool = True, p_num: int = 24,
                 t_num: int = 8, max_iter: int = 1000, precision: str = "fp64", solver: PointSolver | None = None,
                 boundary_path: str | None = None, cep_path: str | None = None) -> dict:
    """run_tmu_scan (TmuScan.jl:120-234): same keyword arguments, CSV, resume and statistics."""
    T_values = list(np.arange(50.0, 200.0 + 1e-9, 10.0)) if T_values is None else list(T_values)
    mu_values = list(np.arange(0.0, 400.0 + 1e-9, 10.0)) if mu_values is None else list(mu_values)
    solver = solver or gpu_point_solver(p_num, t_num, precision)
    d = os.path.dirname(output_path)
    if d:
        os.makedirs(d, exist_ok=True)
    completed = _tmu_load_completed(output_path) if (resume and not overwrite and os.path.isfile(output_path)) else set()
    mode = "w" if (overwrite or not os.path.isfile(output_path)) else "a"
    rows, stats = tmu_scan_rows(T_values, mu_values, xi_values, solver, use_phase_aware=use_phase_aware,
                                max_iter=max_iter, boundary_path=boundary_path, cep_path=cep_path, skip=completed)
    with open(output_path, mode) as fh:
        if mode == "w":
            fh.write(",".join(TMU_HEADER) + "\n")
        for T, mu, xi, r, msg in rows:
            fh.write(format_tmu_row(T, mu, xi, r, msg) + "\n")
    return dict(stats, output=output_path)
