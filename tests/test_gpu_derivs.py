"""Implicit derivatives of solved states on the GPU (pnjl_derivs_batch), against the oracle
(seven-variable jets: the reference's nested forward-mode AD) and the reference's own golden
values (tests/unit/relaxtime/test_bulk_viscosity_derivatives.jl: T = 150 MeV, mu_B = 800 MeV).

Tolerance against the oracle: 1e-9 of each field's scale (both are exact derivatives in FP64;
the 5 x 5 solve for dx/dtheta amplifies rounding by the Hessian's condition number); 1e-7 for
the four ratios of differences of products (dP/deps|n, dP/dn|eps, v_n^2, dmu_B/dT|sigma),
whose denominators cancel to a few digits at some points and amplify the same rounding.
"""
import numpy as np
import pytest

from julia_relaxtime_gb300 import _capi as api
from julia_relaxtime_gb300 import derivatives as td
from julia_relaxtime_gb300.engine import SolveOptions
from julia_relaxtime_gb300.pnjl import multiseed_table
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
HBARC = 197.327
SCALARS = ("s", "n_B", "ds_dT", "ds_dmu", "dn_dT", "dn_dmu", "pressure", "dP_dT", "dP_dmu", "energy", "deps_dT",
           "deps_dmu", "dP_deps_n", "dP_dn_eps", "v_n_sq", "dmuB_dT_sigma")
RATIOS = ("dP_deps_n", "dP_dn_eps", "v_n_sq", "dmuB_dT_sigma")


def test_bulk_viscosity_golden_point(engine_factory):
    eng = engine_factory(64, 8)
    T = 150.0 / HBARC
    mu = 800.0 / 3.0 / HBARC
    bv = td.bulk_viscosity_coefficients(T, mu, engine=eng)
    assert bv["v_n_sq"] == pytest.approx(0.098640, rel=1e-4)
    assert bv["dμB_dT_sigma"] == pytest.approx(9.543024, rel=1e-4)
    assert bv["dM_dμB"][0] == pytest.approx(-1.053308, rel=1e-4)
    assert bv["dM_dT"][0] == pytest.approx(bv["dM_dT"][1], rel=1e-6)
    args = (bv["masses"][0], mu, T, bv["v_n_sq"], bv["dμB_dT_sigma"], bv["dM_dT"][0], bv["dM_dμB"][0])
    assert td.compute_B_bracket(1.0, *args) == pytest.approx(-1.203043, rel=1e-4)
    assert td.compute_B_bracket(1.0, *args, is_antiquark=True) == pytest.approx(-0.519924, rel=1e-4)
    th = td.thermo_derivatives(T, mu, engine=eng)
    assert th["converged"]
    assert th["entropy"] == pytest.approx(th["dP_dT"], rel=1e-6)
    assert th["rho"] == pytest.approx(th["dP_dmu"] / 3.0, rel=1e-6)
    md = td.mass_derivatives(T, mu, engine=eng)
    np.testing.assert_array_equal(md["dM_dT"], bv["dM_dT"])
    with pytest.raises(NotImplementedError):
        td.mass_derivatives(T, mu, order=2, engine=eng)


@pytest.mark.parametrize("p_num,t_num", [(24, 8), (64, 16)])
def test_derivatives_match_oracle(engine_factory, p_num, t_num):
    eng = engine_factory(p_num, t_num)
    nd = orc.Nodes(p_num, t_num)
    P = orc.default_params()
    rng = np.random.default_rng(p_num + t_num)
    n = 60
    T = rng.uniform(40, 300, n) / HBARC
    mu = rng.uniform(0, 420, n) / HBARC
    xi = rng.uniform(-0.5, 0.5, n)
    table, hot = multiseed_table(4)
    res = eng.solve(T, mu, xi, seed_table=table, seed_table_hot=hot, opts=SolveOptions(iterations=40, ftol=1e-12))
    ok = res["converged"]
    assert ok.mean() > 0.95
    got = eng.derivs(res["x"][ok], T[ok], mu[ok], xi[ok])
    refs = [orc.thermo_derivs(P, nd, res["x"][i], mu[i], T[i], xi[i]) for i in np.flatnonzero(ok)]
    for k in ("dx_dT", "dx_dmu", "dM_dT", "dM_dmu") + SCALARS:
        ref = np.array([r[k] for r in refs])
        scale = np.maximum(np.abs(ref), np.abs(ref).max(axis=0) * 1e-3)
        err = np.abs(got[k] - ref) / scale
        tol = 1e-7 if k in RATIOS else 1e-9
        assert err.max() <= tol, (k, err.max(), int(np.argmax(err.max(axis=-1) if err.ndim > 1 else err)))


def test_derivatives_device_entry_point(engine_factory):
    torch = pytest.importorskip("torch")
    eng = engine_factory(16, 4)
    rng = np.random.default_rng(3)
    n = 200
    T = rng.uniform(50, 300, n) / HBARC
    mu = rng.uniform(0, 400, n) / HBARC
    xi = rng.uniform(-0.4, 0.4, n)
    table, hot = multiseed_table(4)
    res = eng.solve(T, mu, xi, seed_table=table, seed_table_hot=hot, opts=SolveOptions(iterations=40, ftol=1e-11))
    host = eng.derivs(res["x"], T, mu, xi)
    dev = torch.device("cuda", 0)
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in
         (("x", res["x"].ravel()), ("T", T), ("mu", mu), ("xi", xi))}
    widths = dict(api.DERIV_FIELDS)
    keys = ("dx_dT", "dM_dmu", "v_n_sq", "energy")
    out = {k: torch.full((n * widths[k],), np.nan, dtype=torch.float64, device=dev) for k in keys}
    torch.cuda.synchronize()
    m = t["mu"].data_ptr()
    eng.derivs_device(n, t["x"].data_ptr(), t["T"].data_ptr(), m, m, m, t["xi"].data_ptr(),
                      {k: v.data_ptr() for k, v in out.items()})
    eng.synchronize()
    for k, v in out.items():
        assert np.array_equal(v.cpu().numpy().reshape(host[k].shape), host[k]), k
    assert eng.derivs(res["x"][:0], T[:0], mu[:0], xi[:0])["s"].size == 0
