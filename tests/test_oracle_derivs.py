"""The oracle's implicit derivatives (ThermoDerivatives.jl) pinned by the reference's own tests.

* tests/unit/relaxtime/test_bulk_viscosity_derivatives.jl:22-131 -- at T = 150 MeV,
  mu_B = 800 MeV (xi = 0, 64 x 8 nodes): v_n^2 = 0.098640, dmu_B/dT|sigma = 9.543024,
  dM_u/dmu_B = -1.053308, and compute_B_bracket at p = 1 fm^-1: -1.203043 (quark),
  -0.519924 (antiquark), all to rtol 1e-4; u and d derivatives equal; the thermodynamic
  identities s = dP/dT, n_B = (1/3) dP/dmu_q (:163-173).
* tests/unit/pnjl/test_thermo_derivatives.jl:33-50 -- dP/dT against a central difference of
  the pressure (here at tight tolerance, and for dx/dT, dx/dmu against central differences of
  the solved states).
"""
import numpy as np
import pytest

from oracle import oracle as orc

HBARC = 197.327


@pytest.fixture(scope="module")
def P():
    return orc.default_params()


def _solve(P, nd, T, mu, x0=None):
    seeds = orc.multiseed_seeds(P, T) if x0 is None else x0
    r = orc.solve_point(P, nd, T, [mu] * 3, 0.0, seeds, x0 is None,
                        orc.default_opts(max_iter=60, ftol=1e-13, xtol=0.0))
    return r


def compute_B_bracket(p, M, mu_q, T, v_n_sq, dmuB_dT_sigma, dM_dT, dM_dmuB, antiquark):
    """ThermoDerivatives.jl:473-494 (the bulk-viscosity B term), restated for the check."""
    E = np.sqrt(p * p + M * M)
    dE_dT = M / E * dM_dT
    dE_dmuB = M / E * dM_dmuB
    if antiquark:
        dx = dE_dT + (dE_dmuB + 1.0 / 3.0) * dmuB_dT_sigma
        x = E + mu_q
    else:
        dx = dE_dT + (dE_dmuB - 1.0 / 3.0) * dmuB_dT_sigma
        x = E - mu_q
    return p * p + 3.0 * v_n_sq * T * T * E * (dx / T - x / T ** 2)


def test_bulk_viscosity_golden_point(P):
    nd = orc.Nodes(64, 8)
    T = 150.0 / HBARC
    mu = 800.0 / 3.0 / HBARC
    r = orc.solve_point(P, nd, T, [mu] * 3, 0.0, orc.multiseed_seeds(P, T), True, orc.default_opts())
    assert r["converged"]
    d = orc.thermo_derivs(P, nd, r["x"], mu, T, 0.0)
    dM_dmuB = d["dM_dmu"] / 3.0
    assert d["v_n_sq"] == pytest.approx(0.098640, rel=1e-4)
    assert d["dmuB_dT_sigma"] == pytest.approx(9.543024, rel=1e-4)
    assert dM_dmuB[0] == pytest.approx(-1.053308, rel=1e-4)
    assert d["dM_dT"][0] == pytest.approx(d["dM_dT"][1], rel=1e-6)
    assert d["s"] > 0 and d["n_B"] > 0
    M = r["masses"][0]
    args = (M, mu, T, d["v_n_sq"], d["dmuB_dT_sigma"], d["dM_dT"][0], dM_dmuB[0])
    assert compute_B_bracket(1.0, *args, antiquark=False) == pytest.approx(-1.203043, rel=1e-4)
    assert compute_B_bracket(1.0, *args, antiquark=True) == pytest.approx(-0.519924, rel=1e-4)
    # s = dP/dT and n_B = (1/3) dP/dmu_q
    assert d["s"] == pytest.approx(d["dP_dT"], rel=1e-6)
    assert d["n_B"] == pytest.approx(d["dP_dmu"] / 3.0, rel=1e-6)


@pytest.mark.parametrize("T_MeV,mu_MeV,xi", [(130.0, 320.0 / 3.0, 0.0), (90.0, 250.0, 0.2), (200.0, 50.0, -0.3)])
def test_derivatives_match_central_differences(P, T_MeV, mu_MeV, xi):
    nd = orc.Nodes(24, 8)
    T, mu = T_MeV / HBARC, mu_MeV / HBARC
    seeds = orc.multiseed_seeds(P, T)
    opts = orc.default_opts(max_iter=60, ftol=1e-13, xtol=0.0)
    r = orc.solve_point(P, nd, T, [mu] * 3, xi, seeds, True, orc.default_opts(max_iter=60))
    assert r["converged"]
    x0 = r["x"]

    def at(Tv, muv):
        rr = orc.solve_point(P, nd, Tv, [muv] * 3, xi, x0, False, opts)
        th = orc.thermo(P, nd, rr["x"], [muv] * 3, Tv, xi)
        return rr["x"], th

    x_c, _ = at(T, mu)
    d = orc.thermo_derivs(P, nd, x_c, mu, T, xi)
    h = 1e-4
    xp, tp = at(T + h, mu)
    xm, tm = at(T - h, mu)
    np.testing.assert_allclose((xp - xm) / (2 * h), d["dx_dT"], rtol=1e-5, atol=1e-7)
    assert (tp["pressure"] - tm["pressure"]) / (2 * h) == pytest.approx(d["dP_dT"], rel=1e-6)
    assert (tp["entropy"] - tm["entropy"]) / (2 * h) == pytest.approx(d["ds_dT"], rel=1e-5)
    xp, tp = at(T, mu + h)
    xm, tm = at(T, mu - h)
    np.testing.assert_allclose((xp - xm) / (2 * h), d["dx_dmu"], rtol=1e-5, atol=1e-7)
    nb = lambda th: sum(th["rho"]) / 3.0  # noqa: E731
    assert (nb(tp) - nb(tm)) / (2 * h) == pytest.approx(d["dn_dmu"], rel=1e-5, abs=1e-9)
    assert (tp["energy"] - tm["energy"]) / (2 * h) == pytest.approx(d["deps_dmu"], rel=1e-5)
