"""Phase structure from batched GPU solves: the dual-branch scan of
src/pnjl/scans/DualBranchScan.jl and the first-order line and CEP data that
PhaseAwareContinuitySeed reads (data/reference/pnjl/boundary.csv, cep.csv).

DualBranchScan.jl follows two branches along mu at fixed T, one point at a time: the hadron
branch upward from the lowest mu (ContinuitySeed with a hadron fallback), the quark branch
downward from the highest (quark fallback); a branch ends where its solve fails or its
solution jumps (|d phi_u| > 0.5 or |d M_u| > 50 MeV); the physical branch is the lower Omega
(DualBranchScan.jl:104-243, 411-470); the transition is the Omega crossing inside the
coexistence region (:253-316, 496-530).  Lines (T, xi) are independent, so here every line
of a scan advances together: step k of a branch solves the k-th mu of every line still
followed in one GPU launch (per-point seeds from each line's tracker, the MultiSeed fallback
of solve), then the trackers are updated exactly as the reference updates them.

The reference builds boundary.csv and cep.csv (scripts/pnjl/calculate_phase_structure.jl)
from T-rho scans with a Maxwell construction; the equal-pressure point of that construction
is the Omega crossing of the two branches, which is what the dual-branch scan finds at fixed
mu.  phase_boundary() writes the same columns -- xi, T_MeV, mu_transition_MeV (the quark
chemical potential at the crossing), rho_hadron, rho_quark (rho / rho0 of the two branches
there) -- and locate_cep() brackets the highest T with a first-order crossing and bisects it.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .constants import HBARC_MEV_FM
from .pnjl import ContinuitySeed, DefaultSeed, FixedMu, default_engine, solve_batch


@dataclass
class BranchPoint:
    """DualBranchScan.jl:49-61."""
    mu_mev: float
    converged: bool
    omega: float
    pressure: float
    rho_norm: float
    entropy: float
    energy: float
    x_state: np.ndarray
    masses: np.ndarray
    iterations: int
    residual_norm: float


@dataclass
class DualBranchResult:
    """DualBranchScan.jl:64-71."""
    T_mev: float
    xi: float
    mu_values: np.ndarray
    hadron_branch: list
    quark_branch: list
    physical_branch: list = field(default_factory=list)


@dataclass
class PhaseTransitionInfo:
    """DualBranchScan.jl:74-81."""
    found: bool
    mu_c: float
    omega_at_transition: float
    mu_hadron_spinodal: float
    mu_quark_spinodal: float
    coexistence_region: tuple


def _is_same_solution(h: BranchPoint, q: BranchPoint, tol: float = 0.01) -> bool:
    """DualBranchScan.jl:443-452."""
    return (abs(h.x_state[0] - q.x_state[0]) < tol and abs(h.x_state[3] - q.x_state[3]) < tol and
            abs(h.masses[0] - q.masses[0]) < tol * 197.327)


def _is_solution_jump(prev_x, prev_m, x, m, phi_threshold: float = 0.5, mass_threshold: float = 50.0) -> bool:
    """DualBranchScan.jl:455-465 (mass change in MeV)."""
    return abs(prev_x[0] - x[0]) > phi_threshold or abs(prev_m[0] - m[0]) * 197.327 > mass_threshold


def _select_physical_branch(hadron, quark):
    """DualBranchScan.jl:411-440."""
    out = []
    for h, q in zip(hadron, quark):
        if h is None and q is None:
            out.append(None)
        elif h is None:
            out.append(q)
        elif q is None:
            out.append(h)
        elif _is_same_solution(h, q):
            out.append(h)
        else:
            out.append(h if h.omega <= q.omega else q)
    return out


def _follow_branches(lines, mu_grid, hadron: bool, solver):
    """One branch for every line: step k solves the k-th mu (ascending for the hadron branch,
    descending for the quark branch) of every line still followed, in one launch.  mu_grid
    [lines, n_mu]: each line's own ascending mu values (MeV)."""
    n_mu = mu_grid.shape[1]
    order = range(n_mu) if hadron else range(n_mu - 1, -1, -1)
    hint = "hadron" if hadron else "quark"
    trackers = [ContinuitySeed(fallback=DefaultSeed(phase_hint=hint)) for _ in lines]
    prev = [None] * len(lines)
    active = list(range(len(lines)))
    branch = [[None] * n_mu for _ in lines]
    for i in order:
        if not active:
            break
        T = np.array([lines[j][0] / HBARC_MEV_FM for j in active])
        xi = np.array([lines[j][1] for j in active])
        mu = np.array([mu_grid[j, i] / HBARC_MEV_FM for j in active])
        seeds = np.array([trackers[j].get_seed([T[k], mu[k]], FixedMu()) for k, j in enumerate(active)])
        res = solver(T, mu, xi, seeds)
        still = []
        for k, j in enumerate(active):
            if not bool(res["converged"][k]):
                continue  # the branch breaks (DualBranchScan.jl:142-146)
            x, m = np.array(res["x"][k]), np.array(res["masses"][k])
            if prev[j] is not None and _is_solution_jump(prev[j][0], prev[j][1], x, m):
                continue  # a jump ends the branch (:131-135)
            branch[j][i] = BranchPoint(float(mu_grid[j, i]), True, float(res["omega"][k]), float(res["pressure"][k]),
                                       float(res["rho_norm"][k]), float(res["entropy"][k]), float(res["energy"][k]),
                                       x, m, int(res["iterations"][k]), float(res["residual_norm"][k]))
            trackers[j].update(x)
            prev[j] = (x, m)
            still.append(j)
        active = still
    return branch


def gpu_branch_solver(p_num: int = 24, t_num: int = 8, engine=None, iterations: int = 1000):
    """The reference's _solve_point (DualBranchScan.jl:383-397): solve(FixedMu(), T, mu; xi,
    seed_strategy = the tracker's seed, p_num, t_num) -- single seed, trust-region and MultiSeed
    fallbacks -- for many points at once."""
    eng = engine or default_engine(p_num, t_num)

    def solver(T, mu, xi, seeds):
        return solve_batch(T, mu, xi, point_seeds=seeds, p_num=p_num, t_num=t_num, iterations=iterations, engine=eng)

    return solver


def run_dual_branch_scans(T_values_mev, mu_range_mev, xi_values=(0.0,), *, p_num: int = 24, t_num: int = 8,
                          solver=None, lines=None, mu_grid=None) -> list[DualBranchResult]:
    """run_dual_branch_scan (DualBranchScan.jl:104-196) for every (T, xi) line at once: the
    grid T_values x xi_values, or the given (T, xi) pairs; all on mu_range, or each line on
    its own row of mu_grid [lines, n_mu] (MeV, ascending)."""
    solver = solver or gpu_branch_solver(p_num, t_num)
    if lines is None:
        lines = [(float(T), float(xi)) for xi in xi_values for T in T_values_mev]
    lines = [(float(T), float(xi)) for T, xi in lines]
    if mu_grid is None:
        mu_grid = np.tile(np.array([float(m) for m in mu_range_mev]), (len(lines), 1))
    mu_grid = np.asarray(mu_grid, dtype=np.float64).reshape(len(lines), -1)
    had = _follow_branches(lines, mu_grid, True, solver)
    qrk = _follow_branches(lines, mu_grid, False, solver)
    out = []
    for j, (T, xi) in enumerate(lines):
        r = DualBranchResult(T, xi, mu_grid[j].copy(), had[j], qrk[j])
        r.physical_branch = _select_physical_branch(r.hadron_branch, r.quark_branch)
        out.append(r)
    return out


def run_dual_branch_scan(T_mev: float, mu_range, xi: float = 0.0, **kw) -> DualBranchResult:
    """run_dual_branch_scan(; T_mev, mu_range, xi, p_num=24, t_num=8) for one line."""
    return run_dual_branch_scans([T_mev], mu_range, [xi], **kw)[0]


def _find_branch_endpoint(branch, mu_values, forward: bool) -> float:
    """DualBranchScan.jl:468-481."""
    idx = range(len(branch) - 1, -1, -1) if forward else range(len(branch))
    for i in idx:
        if branch[i] is not None:
            return float(mu_values[i])
    return float("nan")


def _find_omega_crossing(mu_vals, om_h, om_q):
    """DualBranchScan.jl:496-530: linear interpolation of the first sign change of
    Omega_hadron - Omega_quark among points whose difference exceeds max(1e-6 |Omega|, 1e-10)."""
    delta = np.asarray(om_h) - np.asarray(om_q)
    sig = [i for i in range(len(mu_vals))
           if abs(delta[i]) > max(1e-6 * 0.5 * (abs(om_h[i]) + abs(om_q[i])), 1e-10)]
    if len(sig) < 2:
        return float("nan"), float("nan")
    for a, b in zip(sig[:-1], sig[1:]):
        if delta[a] * delta[b] < 0:
            t = delta[a] / (delta[a] - delta[b])
            return mu_vals[a] + t * (mu_vals[b] - mu_vals[a]), om_h[a] + t * (om_h[b] - om_h[a])
    return float("nan"), float("nan")


def find_phase_transition(result: DualBranchResult, same_tol: float = 0.01) -> PhaseTransitionInfo:
    """DualBranchScan.jl:253-316 (same_tol: _is_same_solution's tolerance, 0.01 there)."""
    mu = result.mu_values
    h, q = result.hadron_branch, result.quark_branch
    mu_hs = _find_branch_endpoint(h, mu, True)
    mu_qs = _find_branch_endpoint(q, mu, False)
    co = [i for i in range(len(mu))
          if h[i] is not None and q[i] is not None and not _is_same_solution(h[i], q[i], same_tol)]
    if not co:
        return PhaseTransitionInfo(False, float("nan"), float("nan"), mu_hs, mu_qs, (float("nan"), float("nan")))
    mu_c, om_c = _find_omega_crossing([mu[i] for i in co], [h[i].omega for i in co], [q[i].omega for i in co])
    return PhaseTransitionInfo(not math.isnan(mu_c), mu_c, om_c, mu_hs, mu_qs, (float(mu[co[0]]), float(mu[co[-1]])))


MERGED_HEADER = ["T_MeV", "mu_MeV", "xi", "branch", "omega", "pressure", "rho", "entropy", "energy", "phi_u", "phi_d",
                 "phi_s", "Phi1", "Phi2", "M_u_MeV", "M_d_MeV", "M_s_MeV", "delta_omega"]


def merge_branches(result: DualBranchResult, output_path: str | None = None) -> list[dict]:
    """DualBranchScan.jl:323-380 (and its CSV writer :533-560: %.6f for T, mu, xi and the
    masses, %.10f for the rest)."""
    rows = []
    for i, mu in enumerate(result.mu_values):
        pt, h, q = result.physical_branch[i], result.hadron_branch[i], result.quark_branch[i]
        if pt is None:
            continue
        if h is not None and q is not None:
            if _is_same_solution(h, q):
                branch = "same"
            elif abs(pt.omega - h.omega) < 1e-10:
                branch = "hadron"
            else:
                branch = "quark"
        elif h is not None:
            branch = "hadron"
        else:
            branch = "quark"
        d_om = h.omega - q.omega if (h is not None and q is not None and not _is_same_solution(h, q)) else float("nan")
        x = pt.x_state
        rows.append(dict(T_MeV=result.T_mev, mu_MeV=float(mu), xi=result.xi, branch=branch, omega=pt.omega,
                         pressure=pt.pressure, rho=pt.rho_norm, entropy=pt.entropy, energy=pt.energy, phi_u=x[0],
                         phi_d=x[1], phi_s=x[2], Phi1=x[3], Phi2=x[4], M_u_MeV=pt.masses[0] * HBARC_MEV_FM,
                         M_d_MeV=pt.masses[1] * HBARC_MEV_FM, M_s_MeV=pt.masses[2] * HBARC_MEV_FM, delta_omega=d_om))
    if output_path is not None:
        six = {"T_MeV", "mu_MeV", "xi", "M_u_MeV", "M_d_MeV", "M_s_MeV"}
        with open(output_path, "w") as fh:
            fh.write(",".join(MERGED_HEADER) + "\n")
            for r in rows:
                vals = []
                for k in MERGED_HEADER:
                    v = r[k]
                    if k == "branch":
                        vals.append(v)
                    elif isinstance(v, float) and math.isnan(v):
                        vals.append("NaN")
                    else:
                        vals.append(("%.6f" if k in six else "%.10f") % v)
                fh.write(",".join(vals) + "\n")
    return rows


def scan_phase_diagram(T_range, mu_range, xi: float = 0.0, **kw) -> list[PhaseTransitionInfo]:
    """scan_phase_diagram (DualBranchScan.jl:566-597): the transition at every T, all T at once."""
    return [find_phase_transition(r) for r in run_dual_branch_scans(list(T_range), mu_range, [xi], **kw)]


def refine_scans(results: list[DualBranchResult], n_fine: int = 161, **kw) -> list[DualBranchResult]:
    """A second, finer dual-branch scan of every line over the window where its branches end
    or coexist (the coarse scan's spinodals, padded by two coarse steps): near the critical
    end point the coexistence region is narrower than a coarse mu step."""
    lines, grids = [], []
    for r in results:
        step = float(r.mu_values[1] - r.mu_values[0]) if r.mu_values.size > 1 else 1.0
        ends = [v for v in (_find_branch_endpoint(r.hadron_branch, r.mu_values, True),
                            _find_branch_endpoint(r.quark_branch, r.mu_values, False)) if not math.isnan(v)]
        if not ends:
            lo, hi = float(r.mu_values[0]), float(r.mu_values[-1])
        else:
            lo = max(float(r.mu_values[0]), min(ends) - 2 * step)
            hi = min(float(r.mu_values[-1]), max(ends) + 2 * step)
        lines.append((r.T_mev, r.xi))
        grids.append(np.linspace(lo, hi, n_fine))
    return run_dual_branch_scans(None, None, lines=lines, mu_grid=np.array(grids), **kw)


def _interp_rho(branch, mu_values, mu_c):
    """rho / rho0 of a branch at mu_c, linear between its two neighbouring points."""
    pts = [(b.mu_mev, b.rho_norm) for b in branch if b is not None]
    if not pts:
        return float("nan")
    m = np.array([p[0] for p in pts])
    r = np.array([p[1] for p in pts])
    return float(np.interp(mu_c, m, r))


def phase_boundary(xi_values, T_values_mev, mu_range_mev, *, n_fine: int = 161, **kw) -> list[dict]:
    """First-order line rows (boundary.csv columns) for every xi and T with a crossing: a
    coarse scan of every line, then a fine one around its spinodals (refine_scans)."""
    rows = []
    coarse = run_dual_branch_scans(T_values_mev, mu_range_mev, xi_values, **kw)
    for r in refine_scans(coarse, n_fine, **kw):
        info = find_phase_transition(r)
        if not info.found:
            continue
        rows.append(dict(xi=r.xi, T_MeV=r.T_mev, mu_transition_MeV=info.mu_c,
                         rho_hadron=_interp_rho(r.hadron_branch, r.mu_values, info.mu_c),
                         rho_quark=_interp_rho(r.quark_branch, r.mu_values, info.mu_c)))
    return rows


def locate_cep(xi_values, mu_range_mev, T_lo_mev: float, T_hi_mev: float, *, tol_mev: float = 0.25,
               n_fine: int = 201, levels: int = 3, same_tol: float = 1e-4, **kw) -> list[dict]:
    """Critical end point per xi: the highest T with a first-order crossing, by bisection
    between T_lo (a crossing) and T_hi (none); mu_CEP is the crossing at the bracket's lower
    end.  All xi are bisected together (one batched coarse + fine scan per step).  Near the
    CEP the two branches differ by little, so they count as distinct down to same_tol (the
    reference's merge tolerance, 0.01, would end the first-order line early)."""
    lo = {xi: float(T_lo_mev) for xi in xi_values}
    hi = {xi: float(T_hi_mev) for xi in xi_values}
    mu_at = {}

    def scan(lines):
        r = run_dual_branch_scans(None, mu_range_mev, lines=lines, **kw)
        for _ in range(levels):  # zoom in on the spinodals: the coexistence window closes at the CEP
            r = refine_scans(r, n_fine, **kw)
        return r

    for r in scan([(T_lo_mev, x) for x in xi_values]):
        info = find_phase_transition(r, same_tol)
        if not info.found:
            raise ValueError(f"no first-order crossing at T = {T_lo_mev} MeV, xi = {r.xi}")
        mu_at[r.xi] = info.mu_c
    while max(hi[x] - lo[x] for x in xi_values) > tol_mev:
        mids = {x: 0.5 * (lo[x] + hi[x]) for x in xi_values}
        res = scan([(mids[x], x) for x in xi_values])
        for x, r in zip(xi_values, res):
            info = find_phase_transition(r, same_tol)
            if info.found:
                lo[x] = mids[x]
                mu_at[x] = info.mu_c
            else:
                hi[x] = mids[x]
    return [dict(xi=x, T_CEP_MeV=lo[x], mu_CEP_MeV=mu_at[x]) for x in xi_values]


def write_boundary_csv(rows, path: str):
    with open(path, "w") as fh:
        fh.write("xi,T_MeV,mu_transition_MeV,rho_hadron,rho_quark\n")
        for r in rows:
            fh.write(f"{r['xi']!r},{r['T_MeV']!r},{r['mu_transition_MeV']!r},{r['rho_hadron']!r},{r['rho_quark']!r}\n")


def write_cep_csv(rows, path: str):
    with open(path, "w") as fh:
        fh.write("xi,T_CEP_MeV,mu_CEP_MeV\n")
        for r in rows:
            fh.write(f"{r['xi']!r},{r['T_CEP_MeV']!r},{r['mu_CEP_MeV']!r}\n")
