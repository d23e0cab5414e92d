"""Thermodynamic derivatives of the gap solution: the API of
src/pnjl/derivatives/ThermoDerivatives.jl on the GPU (pnjl_derivs_batch).

The reference differentiates the solution x(theta) of the gap equations, theta = (T, mu)
with mu_u = mu_d = mu_s = mu, by the implicit function theorem (ImplicitDifferentiation.jl)
and ForwardDiff; here dx/dtheta = -(Hessian_x Omega)^-1 d(grad_x Omega)/dtheta comes from
analytic second derivatives on the GPU, for any number of points at once.  Each function
first solves (T, mu) as the reference does -- solve(FixedMu(), T, mu; xi, p_num, t_num) with
the default seed strategy -- then differentiates.  Only first derivatives are provided
(mass_derivatives(...; order=2) raises NotImplementedError).
"""
from __future__ import annotations

import numpy as np

from .pnjl import DefaultSeed, FixedMu, default_engine, solve_batch

DEFAULT_MOMENTUM_COUNT = 64  # Integrals.jl:53-54 (GaussLegendre.jl:121-122)
DEFAULT_THETA_COUNT = 8
# compute_masses_from_state (ThermoDerivatives.jl:114-124) uses its own current masses, in
# GeV / (GeV fm): 5.5 MeV and 140 MeV (the model profile has 140.7 MeV for m_s); the masses
# these functions report follow it, the derivatives do not depend on them
_M_U0 = 0.0055 / 0.197327
_M_S0 = 0.140 / 0.197327


def _masses_from_state(engine, x):
    G, K = engine.params.G, engine.params.K
    x = np.asarray(x, dtype=np.float64).reshape(-1, 5)
    pu, pd, ps = x[:, 0], x[:, 1], x[:, 2]
    return np.stack([_M_U0 - 4 * G * pu + 2 * K * pd * ps, _M_U0 - 4 * G * pd + 2 * K * pu * ps,
                     _M_S0 - 4 * G * ps + 2 * K * pu * pd], axis=1)


def derivatives_batch(T_fm, mu_fm, xi=0.0, *, x=None, p_num: int = DEFAULT_MOMENTUM_COUNT,
                      t_num: int = DEFAULT_THETA_COUNT, engine=None, iterations: int = 1000):
    """Solve n points (unless their solutions x [n,5] are given) and differentiate them.
    Returns (solve result or None, derivative arrays: engine.derivs)."""
    eng = engine or default_engine(p_num, t_num)
    eng.set_nodes(p_num, t_num)
    T = np.atleast_1d(np.asarray(T_fm, dtype=np.float64))
    n = T.size
    mu = np.broadcast_to(np.asarray(mu_fm, dtype=np.float64), (n,)).copy()
    xia = np.broadcast_to(np.asarray(xi, dtype=np.float64), (n,)).copy()
    res = None
    if x is None:
        ds = DefaultSeed()
        seeds = np.array([ds.get_seed([T[i], mu[i]], FixedMu()) for i in range(n)])
        res = solve_batch(T, mu, xia, point_seeds=seeds, p_num=p_num, t_num=t_num, iterations=iterations,
                          engine=eng)
        x = res["x"]
    return res, eng.derivs(x, T, mu, xia)


def _one(T_fm, mu_fm, xi, p_num, t_num, engine):
    res, d = derivatives_batch([T_fm], [mu_fm], [xi], p_num=p_num, t_num=t_num, engine=engine)
    return res, {k: (v[0] if v.ndim == 1 else v[0].copy()) for k, v in d.items()}


def mass_derivatives(T_fm: float, mu_fm: float, *, order: int = 1, xi: float = 0.0,
                     p_num: int = DEFAULT_MOMENTUM_COUNT, t_num: int = DEFAULT_THETA_COUNT, engine=None) -> dict:
    """ThermoDerivatives.jl:132-173: masses, dM/dT, dM/dmu (order 1)."""
    if order != 1:
        raise NotImplementedError("only first derivatives are computed on the GPU (order=1)")
    res, d = _one(T_fm, mu_fm, xi, p_num, t_num, engine)
    eng = engine or default_engine(p_num, t_num)
    return dict(masses=_masses_from_state(eng, res["x"][0])[0], dM_dT=d["dM_dT"], dM_dmu=d["dM_dmu"])


def thermo_derivatives(T_fm: float, mu_fm: float, *, xi: float = 0.0, p_num: int = DEFAULT_MOMENTUM_COUNT,
                       t_num: int = DEFAULT_THETA_COUNT, engine=None) -> dict:
    """ThermoDerivatives.jl:184-249: P, eps, n, s with their T and mu derivatives, dP/deps|n,
    dP/dn|eps, the masses with their derivatives, and the solve's status."""
    res, d = _one(T_fm, mu_fm, xi, p_num, t_num, engine)
    eng = engine or default_engine(p_num, t_num)
    return dict(pressure=d["pressure"], energy=d["energy"], rho=d["n_B"], rho_norm=float(res["rho_norm"][0]),
                entropy=d["s"], dP_dT=d["dP_dT"], dP_dmu=d["dP_dmu"], dEpsilon_dT=d["deps_dT"],
                dEpsilon_dmu=d["deps_dmu"], dn_dT=d["dn_dT"], dn_dmu=d["dn_dmu"], dP_depsilon_n=d["dP_deps_n"],
                dP_dn_epsilon=d["dP_dn_eps"], masses=_masses_from_state(eng, res["x"][0])[0], dM_dT=d["dM_dT"],
                dM_dmu=d["dM_dmu"], converged=bool(res["converged"][0]), iterations=int(res["iterations"][0]),
                residual_norm=float(res["residual_norm"][0]))


def bulk_derivative_coeffs(T_fm: float, mu_fm: float, **kw) -> dict:
    """ThermoDerivatives.jl:256-264."""
    t = thermo_derivatives(T_fm, mu_fm, **kw)
    return dict(dP_depsilon_n=t["dP_depsilon_n"], dP_dn_epsilon=t["dP_dn_epsilon"], dM_dT=t["dM_dT"],
                dM_dmu=t["dM_dmu"])


def dP_dT(T_fm: float, mu_fm: float, *, order: int = 1, **kw) -> float:
    """ThermoDerivatives.jl:279-295 (order 1)."""
    if order != 1:
        raise NotImplementedError("only order=1 is computed on the GPU")
    return thermo_derivatives(T_fm, mu_fm, **kw)["dP_dT"]


def dP_dmu(T_fm: float, mu_fm: float, *, order: int = 1, **kw) -> float:
    """ThermoDerivatives.jl:302-318 (order 1)."""
    if order != 1:
        raise NotImplementedError("only order=1 is computed on the GPU")
    return thermo_derivatives(T_fm, mu_fm, **kw)["dP_dmu"]


def bulk_viscosity_coefficients(T_fm: float, mu_fm: float, *, xi: float = 0.0,
                                p_num: int = DEFAULT_MOMENTUM_COUNT, t_num: int = DEFAULT_THETA_COUNT,
                                engine=None) -> dict:
    """ThermoDerivatives.jl:342-465: v_n^2, dmu_B/dT at fixed s/n_B, masses, dM/dT, dM/dmu_B,
    s and n_B."""
    res, d = _one(T_fm, mu_fm, xi, p_num, t_num, engine)
    eng = engine or default_engine(p_num, t_num)
    return {"v_n_sq": d["v_n_sq"], "dμB_dT_sigma": d["dmuB_dT_sigma"],
            "masses": _masses_from_state(eng, res["x"][0])[0], "dM_dT": d["dM_dT"], "dM_dμB": d["dM_dmu"] / 3.0,
            "s": d["s"], "n_B": d["n_B"]}


def compute_B_bracket(p: float, M: float, mu_q: float, T: float, v_n_sq: float, dmuB_dT_sigma: float,
                      dM_dT: float, dM_dmuB: float, *, is_antiquark: bool = False) -> float:
    """ThermoDerivatives.jl:473-494: the B term of the bulk-viscosity formula."""
    E = np.sqrt(p * p + M * M)
    dE_dT = (M / E) * dM_dT
    dE_dmuB = (M / E) * dM_dmuB
    b_q = 1.0 / 3.0
    if is_antiquark:
        dx = dE_dT + (dE_dmuB + b_q) * dmuB_dT_sigma
        x = E + mu_q
    else:
        dx = dE_dT + (dE_dmuB - b_q) * dmuB_dT_sigma
        x = E - mu_q
    return p * p + 3.0 * v_n_sq * T * T * E * (dx / T - x / T ** 2)
