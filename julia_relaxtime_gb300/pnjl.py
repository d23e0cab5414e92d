"""The reference's PNJL solver API, mirrored in Python over libpnjl_cuda.

Julia (w5851/Julia_RelaxTime, src/pnjl/PNJL.jl)        here
-------------------------------------------------      ---------------------------------------
solve(FixedMu(), T_fm, mu_fm; xi, seed_strategy, ...)  solve(FixedMu(), T_fm, mu_fm, xi=..., ...)
solve_multi(FixedMu(), T_fm, mu_fm; seed_strategy)     solve_multi(...)
SolverResult                                           SolverResult (same fields)
SeedStrategy, DefaultSeed, MultiSeed, ContinuitySeed,  same classes; update!/reset!/set_phase!
PhaseAwareContinuitySeed, get_seed, get_all_seeds       are update()/reset()/set_phase()
HADRON_SEED_5, QUARK_SEED_5, ...                       same constants
(new) solve_batch(T, mu, xi; seed_strategy)            one GPU launch for many points

Every solve runs on the GPU through GapEngine; there is no CPU path.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from typing import Callable, Sequence

import numpy as np

from . import _capi as api
from .constants import HBARC_MEV_FM, PNJLParams

# ---------------------------------------------------------------------------------------
# Built-in seeds (SeedStrategies.jl:56-95): (phi_u, phi_d, phi_s, Phi, Phibar)
HADRON_SEED_5 = (-1.84329, -1.84329, -2.22701, 1.0e-5, 4.0e-5)
MEDIUM_SEED_5 = (-1.3647, -1.3647, -2.14502, 0.10594, 0.15569)
HIGH_DENSITY_SEED_5 = (-0.21695, -0.21695, -2.01372, 0.18601, 0.22333)
HIGH_TEMP_SEED_5 = (-0.73192, -0.73192, -1.79539, 0.60532, 0.60532)
VERY_HIGH_TEMP_SEED_5 = (-0.30, -0.30, -0.90, 0.90, 0.90)
HT_GUESS_0p8_SEED_5 = (-0.50, -0.50, -1.20, 0.80, 0.80)
HT_GUESS_0p9_SEED_5 = (-0.30, -0.30, -0.90, 0.90, 0.90)
HT_GUESS_0p95_SEED_5 = (-0.20, -0.20, -0.70, 0.95, 0.95)
WEAK_CHIRAL_CONF_SEED_5 = (-0.50, -0.50, -1.20, 1e-3, 1e-3)
QUARK_SEED_5 = HIGH_TEMP_SEED_5

HOT_T_MEV = 300.0  # DefaultSeed(:quark) switches to VERY_HIGH_TEMP at T >= 300 MeV (SeedStrategies.jl:212-220)


class ConstraintMode:
    pass


class FixedMu(ConstraintMode):
    """Fixed chemical potential mode (ConstraintModes.jl:48); state x = (phi_u, phi_d, phi_s, Phi, Phibar)."""

    def __repr__(self):
        return "FixedMu()"


def state_dim(mode: ConstraintMode) -> int:
    if isinstance(mode, FixedMu):
        return 5
    raise NotImplementedError("only FixedMu is on the GPU path")


def auto_phase_hint(T_fm: float, mu_fm: float) -> str:
    """SeedStrategies.jl:131-136: quark when T > 150 MeV or mu > 300 MeV."""
    return "quark" if (T_fm * 197.327 > 150 or mu_fm * 197.327 > 300) else "hadron"


def extend_seed(base, mode: ConstraintMode) -> np.ndarray:
    if isinstance(mode, FixedMu):
        return np.array(base[:5], dtype=np.float64)
    raise NotImplementedError


# ---------------------------------------------------------------------------------------
class SeedStrategy:
    """Abstract initial-guess strategy (SeedStrategies.jl:118)."""

    def get_seed(self, theta: Sequence[float], mode: ConstraintMode) -> np.ndarray:
        raise NotImplementedError


@dataclass
class DefaultSeed(SeedStrategy):
    """SeedStrategies.jl:188-225."""
    hadron_seed: tuple = HADRON_SEED_5
    quark_seed: tuple = QUARK_SEED_5
    phase_hint: str = "auto"

    def get_seed(self, theta, mode):
        hint = self.phase_hint
        if hint == "auto":
            hint = auto_phase_hint(theta[0], theta[1]) if len(theta) >= 2 else "hadron"
        if hint == "quark":
            base = self.quark_seed
            if len(theta) >= 1 and theta[0] * 197.327 >= HOT_T_MEV:
                base = VERY_HIGH_TEMP_SEED_5
        else:
            base = self.hadron_seed
        return extend_seed(base, mode)

    def __repr__(self):
        return f"DefaultSeed(phase_hint={self.phase_hint})"


def default_omega_selector(results):
    """SeedStrategies.jl:236-240: the converged result with the smallest Omega (first minimum)."""
    conv = [r for r in results if r.converged]
    if not conv:
        return results[0]
    best = conv[0]
    for r in conv[1:]:
        if r.omega < best.omega:
            best = r
    return best


@dataclass
class MultiSeed(SeedStrategy):
    """SeedStrategies.jl:254-284: six candidates, min-Omega selection."""
    candidates: list = field(default_factory=lambda: [
        DefaultSeed(phase_hint="hadron"),
        DefaultSeed(phase_hint="quark"),
        DefaultSeed(WEAK_CHIRAL_CONF_SEED_5, WEAK_CHIRAL_CONF_SEED_5, "hadron"),
        DefaultSeed(HT_GUESS_0p8_SEED_5, HT_GUESS_0p8_SEED_5, "hadron"),
        DefaultSeed(HT_GUESS_0p9_SEED_5, HT_GUESS_0p9_SEED_5, "hadron"),
        DefaultSeed(HT_GUESS_0p95_SEED_5, HT_GUESS_0p95_SEED_5, "hadron"),
    ])
    selector: Callable = default_omega_selector

    def get_seed(self, theta, mode):
        return self.candidates[0].get_seed(theta, mode)

    def get_all_seeds(self, theta, mode):
        return [c.get_seed(theta, mode) for c in self.candidates]

    def tables(self):
        """(table, hot_table) for the GPU: candidate seeds at T < 300 MeV and at T >= 300 MeV."""
        if any(getattr(c, "phase_hint", None) == "auto" for c in self.candidates):
            raise ValueError("auto-hint candidates depend on mu; pass per-point seeds instead")
        t_hot = HOT_T_MEV / HBARC_MEV_FM * (1 + 1e-12)
        cold = np.array([c.get_seed([0.0, 0.0], FixedMu()) for c in self.candidates])
        hot = np.array([c.get_seed([t_hot, 0.0], FixedMu()) for c in self.candidates])
        return np.ascontiguousarray(cold), np.ascontiguousarray(hot)

    def __repr__(self):
        return f"MultiSeed({len(self.candidates)} candidates)"


def multiseed_table(n: int = 6, extra: Sequence[tuple] = ()):
    """Seed table of MultiSeed() (first n candidates), plus extra rows, for the GPU."""
    cold, hot = MultiSeed().tables()
    cold, hot = cold[:n], hot[:n]
    if extra:
        ex = np.array(extra, dtype=np.float64).reshape(-1, 5)
        cold = np.vstack([cold, ex])
        hot = np.vstack([hot, ex])
    return np.ascontiguousarray(cold), np.ascontiguousarray(hot)


def get_all_seeds(s: MultiSeed, theta, mode):
    return s.get_all_seeds(theta, mode)


def get_seed(s: SeedStrategy, theta, mode):
    return s.get_seed(theta, mode)


@dataclass
class ContinuitySeed(SeedStrategy):
    """SeedStrategies.jl:300-345."""
    previous_solution: np.ndarray | None = None
    fallback: SeedStrategy = field(default_factory=DefaultSeed)

    def get_seed(self, theta, mode):
        if self.previous_solution is not None and len(self.previous_solution) >= 5:
            return extend_seed(self.previous_solution, mode)
        return self.fallback.get_seed(theta, mode)

    def update(self, solution, *_):
        self.previous_solution = np.array(solution, dtype=np.float64)
        return self

    def reset(self):
        self.previous_solution = None
        return self


# ---------------------------------------------------------------------------------------
@dataclass
class PhaseBoundaryData:
    """SeedStrategies.jl:365-380: first-order line mu_c(T) (MeV) and the CEP of one xi."""
    T_values: np.ndarray
    mu_values: np.ndarray
    T_CEP: float
    mu_CEP: float
    xi: float


_BOUNDARY_CACHE: dict = {}


def _file_stamp(path: str):
    try:
        st = os.stat(path)
        return st.st_mtime_ns, st.st_size
    except OSError:
        return None


def load_phase_boundary(xi: float, boundary_path: str, cep_path: str) -> PhaseBoundaryData:
    """SeedStrategies.jl:388-436 (rows with |xi_row - xi| <= 1e-6; sorted by T).  Parsed files
    are kept by path, modification time and size (a scan makes one tracker per column); the
    returned data is shared and read-only."""
    key = (float(xi), boundary_path, cep_path, _file_stamp(boundary_path), _file_stamp(cep_path))
    data = _BOUNDARY_CACHE.get(key)
    if data is None:
        data = _BOUNDARY_CACHE[key] = _read_phase_boundary(xi, boundary_path, cep_path)
    return data


def _read_phase_boundary(xi: float, boundary_path: str, cep_path: str) -> PhaseBoundaryData:
    T_CEP = mu_CEP = float("nan")
    if os.path.isfile(cep_path):
        for line in open(cep_path):
            if line.startswith("xi"):
                continue
            parts = line.strip().split(",")
            if len(parts) < 3:
                continue
            try:
                xv = float(parts[0])
            except ValueError:
                continue
            if abs(xv - xi) > 1e-6:
                continue
            T_CEP, mu_CEP = float(parts[1]), float(parts[2])
            break
    Ts, mus = [], []
    if os.path.isfile(boundary_path):
        for line in open(boundary_path):
            if line.startswith("xi"):
                continue
            parts = line.strip().split(",")
            if len(parts) < 3:
                continue
            try:
                xv, tv, mv = float(parts[0]), float(parts[1]), float(parts[2])
            except ValueError:
                continue
            if abs(xv - xi) > 1e-6:
                continue
            Ts.append(tv)
            mus.append(mv)
    order = np.argsort(np.array(Ts), kind="stable") if Ts else np.array([], dtype=int)
    return PhaseBoundaryData(np.array(Ts)[order], np.array(mus)[order], T_CEP, mu_CEP, float(xi))


def interpolate_mu_c(data: PhaseBoundaryData, T_MeV: float) -> float:
    """SeedStrategies.jl:446-475: linear interpolation, clamped extrapolation, NaN above T_CEP."""
    if not math.isnan(data.T_CEP) and T_MeV > data.T_CEP:
        return float("nan")
    Ts, ms = data.T_values, data.mu_values
    if Ts.size == 0:
        return float("nan")
    if T_MeV <= Ts[0]:
        return float(ms[0])
    if T_MeV >= Ts[-1]:
        return float(ms[-1])
    for i in range(Ts.size - 1):
        if Ts[i] <= T_MeV <= Ts[i + 1]:
            t = (T_MeV - Ts[i]) / (Ts[i + 1] - Ts[i])
            return float(ms[i] + t * (ms[i + 1] - ms[i]))
    return float("nan")


class PhaseAwareContinuitySeed(SeedStrategy):
    """SeedStrategies.jl:679-889: continuation along a scan that switches to the default seed
    of the new phase when the point crosses the first-order line mu_c(T) below the CEP."""

    def __init__(self, xi: float | None = None, *, boundary_path: str | None = None, cep_path: str | None = None,
                 bootstrap_multiseed: bool = False, bootstrap_strategy: MultiSeed | None = None):
        self.boundary_data = None
        if xi is not None and boundary_path is not None and cep_path is not None:
            try:
                self.boundary_data = load_phase_boundary(xi, boundary_path, cep_path)
            except Exception:  # the reference warns and falls back to plain continuation
                self.boundary_data = None
        self.previous_solution = None
        self.previous_phase = "unknown"
        self.hadron_seed = HADRON_SEED_5
        self.quark_seed = QUARK_SEED_5
        self.bootstrap_multiseed = bool(bootstrap_multiseed)
        self.bootstrap_strategy = bootstrap_strategy or MultiSeed()
        self.fallback = DefaultSeed(phase_hint="auto")

    def current_phase(self, T_MeV: float, mu_MeV: float) -> str:
        d = self.boundary_data
        if d is None:
            return "unknown"
        if not math.isnan(d.T_CEP) and T_MeV > d.T_CEP:
            return "crossover"
        mu_c = interpolate_mu_c(d, T_MeV)
        if math.isnan(mu_c):
            return "unknown"
        return "hadron" if mu_MeV < mu_c else "quark"

    def get_seed(self, theta, mode):
        T_MeV = theta[0] * HBARC_MEV_FM
        mu_MeV = (theta[1] if len(theta) >= 2 else 0.0) * HBARC_MEV_FM
        cur = self.current_phase(T_MeV, mu_MeV)
        if self.previous_solution is None:
            if cur == "hadron":
                return extend_seed(self.hadron_seed, mode)
            if cur == "quark":
                return extend_seed(self.quark_seed, mode)
            return self.fallback.get_seed(theta, mode)
        prev = self.previous_phase
        if (prev, cur) in (("hadron", "quark"), ("quark", "hadron")):
            return extend_seed(self.hadron_seed if cur == "hadron" else self.quark_seed, mode)
        return extend_seed(self.previous_solution, mode)

    def update(self, solution, T_MeV: float | None = None, mu_MeV: float | None = None):
        self.previous_solution = np.array(solution, dtype=np.float64)
        if T_MeV is not None and mu_MeV is not None:
            self.previous_phase = self.current_phase(T_MeV, mu_MeV)
        return self

    def reset(self):
        self.previous_solution = None
        self.previous_phase = "unknown"
        return self

    def set_phase(self, phase: str):
        self.previous_phase = phase
        return self


def update(s, *args):
    return s.update(*args)


def reset(s):
    return s.reset()


# ---------------------------------------------------------------------------------------
@dataclass
class SolverResult:
    """ImplicitSolver.jl:178-193 (plus the densities the scan writes)."""
    mode: ConstraintMode
    converged: bool
    solution: np.ndarray
    x_state: np.ndarray
    mu_vec: np.ndarray
    omega: float
    pressure: float
    rho_norm: float
    entropy: float
    energy: float
    masses: np.ndarray
    iterations: int
    residual_norm: float
    xi: float
    rho: np.ndarray = None
    n_q: np.ndarray = None
    n_aq: np.ndarray = None
    status: int = 0
    chosen_seed: int = -1


def _result_at(res, i: int, mode, mu_vec, xi) -> SolverResult:
    x = np.array(res["x"][i])
    return SolverResult(mode=mode, converged=bool(res["converged"][i]), solution=x.copy(), x_state=x,
                        mu_vec=np.array(mu_vec, dtype=np.float64), omega=float(res["omega"][i]),
                        pressure=float(res["pressure"][i]), rho_norm=float(res["rho_norm"][i]),
                        entropy=float(res["entropy"][i]), energy=float(res["energy"][i]),
                        masses=np.array(res["masses"][i]), iterations=int(res["iterations"][i]),
                        residual_norm=float(res["residual_norm"][i]), xi=float(xi), rho=np.array(res["rho"][i]),
                        n_q=np.array(res["n_q"][i]), n_aq=np.array(res["n_aq"][i]), status=int(res["status"][i]),
                        chosen_seed=int(res["chosen_seed"][i]))


class AllSeedsFailed(RuntimeError):
    """solve_multi's error("All seeds failed to converge to a physical solution")."""


class SolverException(RuntimeError):
    """NLsolve raised (non-finite residual at the initial guess)."""


_ENGINES: dict = {}


def default_engine(p_num: int = 64, t_num: int = 8, device: int = 0, params: PNJLParams | None = None):
    """One GapEngine per (device, params) in this process; nodes are switched on demand."""
    from .engine import GapEngine

    key = (device, params)
    eng = _ENGINES.get(key)
    if eng is None:
        eng = GapEngine(params=params, device=device, p_num=p_num, t_num=t_num)
        _ENGINES[key] = eng
    eng.set_nodes(p_num, t_num)
    return eng


def _opts(iterations, trust_region_fallback, auto_multiseed_fallback, residual_norm_max, precision, ftol=1e-9,
          xtol=1e-9, phi_tol=1e-8, omega_tie_rtol=1e-12):
    from .engine import SolveOptions

    return SolveOptions(iterations=iterations, ftol=ftol, xtol=xtol, residual_norm_max=residual_norm_max,
                        phi_tol=phi_tol, omega_tie_rtol=omega_tie_rtol, trust_region_fallback=trust_region_fallback,
                        auto_multiseed_fallback=auto_multiseed_fallback, precision=precision)


def solve_batch(T_fm, mu_fm, xi=0.0, *, seed_strategy: SeedStrategy | None = None, point_seeds=None,
                p_num: int = 64, t_num: int = 8, iterations: int = 1000, trust_region_fallback: bool = True,
                auto_multiseed_fallback: bool = True, residual_norm_max: float = 1e-6, precision: str = "fp64",
                ftol: float = 1e-9, xtol: float = 1e-9, omega_tie_rtol: float = 1e-12, engine=None,
                multiseed: MultiSeed | None = None):
    """Solve many (T, mu, xi) points in one launch.

    mu_fm: [n] (mu_u = mu_d = mu_s) or [n,3].  seed_strategy MultiSeed (default) runs every
    candidate with min-Omega selection; point_seeds [n,5] runs one seed per point with the
    MultiSeed fallback (auto_multiseed_fallback).  Returns the BatchResult arrays.
    """
    eng = engine or default_engine(p_num, t_num)
    if engine is not None:
        eng.set_nodes(p_num, t_num)
    ms = multiseed or (seed_strategy if isinstance(seed_strategy, MultiSeed) else MultiSeed())
    table, hot = ms.tables()
    opts = _opts(iterations, trust_region_fallback, auto_multiseed_fallback, residual_norm_max, precision, ftol,
                 xtol, omega_tie_rtol=omega_tie_rtol)
    if point_seeds is None and seed_strategy is not None and not isinstance(seed_strategy, MultiSeed):
        T_arr = np.atleast_1d(np.asarray(T_fm, dtype=np.float64))
        mu_arr = np.asarray(mu_fm, dtype=np.float64)
        mu1 = mu_arr if mu_arr.ndim <= 1 else mu_arr[:, 0]
        mu1 = np.broadcast_to(mu1, T_arr.shape)
        point_seeds = np.array([seed_strategy.get_seed([T_arr[i], mu1[i]], FixedMu()) for i in range(T_arr.size)])
    return eng.solve(T_fm, mu_fm, xi, seed_table=table, seed_table_hot=hot, hot_T_MeV=HOT_T_MEV,
                     point_seeds=point_seeds, opts=opts)


def solve_multi(mode: FixedMu, T_fm: float, mu_fm: float, *, seed_strategy: MultiSeed | None = None, xi: float = 0.0,
                p_num: int = 64, t_num: int = 8, iterations: int = 1000, trust_region_fallback: bool = True,
                residual_norm_max: float = 1e-6, precision: str = "fp64", engine=None, **_):
    """ImplicitSolver.jl:532-559 on the GPU; raises AllSeedsFailed like the reference."""
    ms = seed_strategy or MultiSeed()
    res = solve_batch(np.array([T_fm]), np.array([mu_fm]), np.array([xi]), seed_strategy=ms, p_num=p_num,
                      t_num=t_num, iterations=iterations, trust_region_fallback=trust_region_fallback,
                      auto_multiseed_fallback=False, residual_norm_max=residual_norm_max, precision=precision,
                      engine=engine)
    if int(res["status"][0]) == api.PNJL_POINT_ALL_SEEDS_FAILED:
        raise AllSeedsFailed("All seeds failed to converge to a physical solution")
    return _result_at(res, 0, mode, [mu_fm] * 3, xi)


def solve(mode: FixedMu, T_fm: float, mu_fm: float, *, xi: float = 0.0, seed_strategy: SeedStrategy | None = None,
          p_num: int = 64, t_num: int = 8, trust_region_fallback: bool = True, auto_multiseed_fallback: bool = True,
          residual_norm_max: float = 1e-6, iterations: int = 1000, precision: str = "fp64", engine=None,
          **_) -> SolverResult:
    """solve(::FixedMu, T_fm, mu_fm; ...) of ImplicitSolver.jl:211-328, on the GPU."""
    if not isinstance(mode, FixedMu):
        raise NotImplementedError("only FixedMu is on the GPU path")
    s = seed_strategy or DefaultSeed()
    if isinstance(s, PhaseAwareContinuitySeed) and s.bootstrap_multiseed and s.previous_solution is None:
        return solve_multi(mode, T_fm, mu_fm, seed_strategy=s.bootstrap_strategy, xi=xi, p_num=p_num, t_num=t_num,
                           iterations=iterations, trust_region_fallback=trust_region_fallback,
                           residual_norm_max=residual_norm_max, precision=precision, engine=engine)
    if isinstance(s, MultiSeed):
        return solve_multi(mode, T_fm, mu_fm, seed_strategy=s, xi=xi, p_num=p_num, t_num=t_num,
                           iterations=iterations, trust_region_fallback=trust_region_fallback,
                           residual_norm_max=residual_norm_max, precision=precision, engine=engine)
    x0 = s.get_seed([T_fm, mu_fm], mode)
    res = solve_batch(np.array([T_fm]), np.array([mu_fm]), np.array([xi]), point_seeds=x0.reshape(1, 5),
                      p_num=p_num, t_num=t_num, iterations=iterations, trust_region_fallback=trust_region_fallback,
                      auto_multiseed_fallback=auto_multiseed_fallback, residual_norm_max=residual_norm_max,
                      precision=precision, engine=engine)
    if int(res["status"][0]) == api.PNJL_POINT_EXCEPTION:
        raise SolverException("non-finite residual at the initial guess")
    return _result_at(res, 0, mode, [mu_fm] * 3, xi)
