"""Parity of the CUDA path (through the C ABI) with the CPU oracle and the golden rows.

Tolerances: FP64 kernel vs the jet-AD oracle -- Omega 1e-13 relative, gradient and Hessian
1e-11 relative (different but exact derivative formulas, rounding only); solved states --
|dphi|/|phi| <= 1e-9 and |dPhi| <= 1e-10 (the required bound), Omega 1e-12 relative.
"""
import os

import numpy as np
import pytest

from julia_relaxtime_gb300 import _capi as api
from julia_relaxtime_gb300 import pnjl
from julia_relaxtime_gb300.engine import SolveOptions
from oracle import oracle as orc
from oracle_adapter import GOLDEN, read_csv

pytestmark = pytest.mark.gpu
HBARC = 197.327


@pytest.fixture(scope="module")
def P():
    return orc.default_params()


def random_states(n, seed, mu_neg=False, asym=False):
    rng = np.random.default_rng(seed)
    T = rng.uniform(20, 350, n) / HBARC
    mu1 = rng.uniform(-200 if mu_neg else 0, 450, n) / HBARC
    mu = np.stack([mu1, mu1, mu1], axis=1)
    if asym:
        mu[:, 1] = mu1 * rng.uniform(0.8, 1.2, n)
        mu[:, 2] = 0.5 * mu1
    xi = rng.uniform(-0.8, 0.8, n)
    x = np.column_stack([rng.uniform(-2.0, -0.05, (n, 3)), rng.uniform(0.0, 1.0, (n, 2))])
    sym = rng.random(n) < 0.5
    x[sym, 1] = x[sym, 0]
    return x, T, mu, xi


@pytest.mark.parametrize("p_num,t_num", [(12, 6), (64, 8), (128, 32), (256, 32)])
def test_nodes_match_oracle(engine_factory, p_num, t_num):
    eng = engine_factory(p_num, t_num)
    p, c, w = eng.nodes()
    nd = orc.Nodes(p_num, t_num)
    np.testing.assert_allclose(p, nd.p, rtol=2e-15, atol=1e-15)
    np.testing.assert_allclose(c, nd.c, rtol=2e-15, atol=1e-16)
    np.testing.assert_allclose(w, nd.w, rtol=2e-14, atol=0)


@pytest.mark.parametrize("p_num,t_num,mu_neg,asym", [(12, 6, False, False), (64, 8, True, False),
                                                     (32, 16, False, True), (128, 32, True, True)])
def test_eval_fp64_matches_oracle(engine_factory, P, p_num, t_num, mu_neg, asym):
    eng = engine_factory(p_num, t_num)
    nd = orc.Nodes(p_num, t_num)
    x, T, mu, xi = random_states(48, p_num + t_num, mu_neg, asym)
    T[:3] = 0.5 / HBARC  # (mu - E)/T beyond the rescaling cap of the FP64 passes
    om, g, h = eng.evaluate(x, T, mu, xi)
    for i in range(len(T)):
        o_ref, g_ref, h_ref = orc.evaluate(P, nd, x[i], mu[i], T[i], xi[i])
        assert abs(om[i] - o_ref) <= 1e-13 * abs(o_ref), (i, om[i], o_ref)
        sg = max(1.0, np.abs(g_ref).max())
        assert np.abs(g[i] - g_ref).max() <= 1e-11 * sg, (i, g[i], g_ref)
        sh = max(1.0, np.abs(h_ref).max())
        assert np.abs(h[i] - h_ref).max() <= 1e-11 * sh, (i, h[i], h_ref)


@pytest.mark.parametrize("mu_neg,asym", [(False, False), (True, True)])
def test_eval_fp32_newton_pass_close_to_fp64(engine_factory, mu_neg, asym):
    """The mixed solver's FP32 Newton pass (regrouped second derivatives, uncompensated
    Jacobian sums): gradient within 1e-5 and Hessian within 1e-4 of their scale of the FP64
    pass (the FP32 resolution of the node sums)."""
    eng = engine_factory(128, 32)
    x, T, mu, xi = random_states(64, 8 + int(mu_neg), mu_neg, asym)
    T = np.maximum(T, 45.0 / HBARC)
    _, g, h = eng.evaluate(x, T, mu, xi)
    _, g32, h32 = eng.evaluate(x, T, mu, xi, precision="fp32_newton")
    for i in range(len(T)):
        sg = max(1.0, np.abs(g[i]).max())
        sh = max(1.0, np.abs(h[i]).max())
        assert np.abs(g32[i] - g[i]).max() <= 1e-5 * sg, (i, g32[i] - g[i])
        assert np.abs(h32[i] - h[i]).max() <= 1e-4 * sh, (i, h32[i] - h[i])


def test_eval_mixed_fp32_pass_close_to_fp64(engine_factory):
    eng = engine_factory(128, 32)
    x, T, mu, xi = random_states(64, 7)
    om, g, h = eng.evaluate(x, T, mu, xi)
    om32, g32, h32 = eng.evaluate(x, T, mu, xi, precision="mixed")
    assert np.abs(om32 - om).max() <= 1e-5 * np.abs(om).max()
    assert np.abs(g32 - g).max() <= 1e-4 * max(1.0, np.abs(g).max())
    assert np.abs(h32 - h).max() <= 1e-4 * max(1.0, np.abs(h).max())


@pytest.mark.parametrize("p_num,t_num,mu_neg,asym", [(64, 8, False, False), (128, 32, True, True)])
def test_eval_ff_residual_matches_oracle(engine_factory, P, p_num, t_num, mu_neg, asym):
    """The float-float passes (FP32 pipe) the mixed solver refines with: gradient to ~1e-12 and
    Hessian to ~1e-11 of their scale, against the FP64 jet oracle (states with mu/T moderate
    enough that no FP32 exponent range is exceeded)."""
    eng = engine_factory(p_num, t_num)
    nd = orc.Nodes(p_num, t_num)
    x, T, mu, xi = random_states(48, 3 + p_num, mu_neg, asym)
    T = np.maximum(T, 45.0 / HBARC)
    _, g, h = eng.evaluate(x, T, mu, xi, precision="ff_residual")
    for i in range(len(T)):
        _, g_ref, h_ref = orc.evaluate(P, nd, x[i], mu[i], T[i], xi[i])
        sg = max(1.0, np.abs(g_ref).max())
        assert np.abs(g[i] - g_ref).max() <= 1e-11 * sg, (i, g[i] - g_ref, sg)
        sh = max(1.0, np.abs(h_ref).max())
        assert np.abs(h[i] - h_ref).max() <= 1e-10 * sh, (i, h[i] - h_ref, sh)


@pytest.mark.parametrize("p_num,t_num,mu_neg,asym", [(64, 8, False, False), (128, 32, True, True)])
def test_eval_fp64_cert_matches_oracle(engine_factory, P, p_num, t_num, mu_neg, asym):
    """The FP64 residual pass that certifies the mixed solver's roots (table exp, hardware
    rcp / rsqrt approximations with Newton corrections): gradient to 1e-12 of its scale
    against the FP64 jet oracle and to 2e-14 against the library-function FP64 pass; states
    at T = 0.5 MeV (exponent arguments below -700: the library exp) included."""
    eng = engine_factory(p_num, t_num)
    nd = orc.Nodes(p_num, t_num)
    x, T, mu, xi = random_states(40, 5 + p_num, mu_neg, asym)
    T[:4] = 0.5 / HBARC
    _, g, _ = eng.evaluate(x, T, mu, xi, precision="fp64_cert")
    _, g64, _ = eng.evaluate(x, T, mu, xi)
    for i in range(len(T)):
        _, g_ref, _ = orc.evaluate(P, nd, x[i], mu[i], T[i], xi[i])
        sg = max(1.0, np.abs(g_ref).max())
        assert np.abs(g[i] - g_ref).max() <= 1e-12 * sg, (i, g[i] - g_ref, sg)
        assert np.abs(g[i] - g64[i]).max() <= 2e-14 * sg, (i, g[i] - g64[i], sg)


def test_f64_math_functions_within_ulps(engine_factory):
    """exp / 1/x / 1/sqrt of the certification pass against correctly rounded references
    (long-double numpy) and the library functions: within 2, 1 and 2 ulp on their fast
    ranges; the arguments outside them give the library function's value."""
    eng = engine_factory(12, 6)
    rng = np.random.default_rng(3)
    ld = np.longdouble

    def ulps(y, ref):
        ref = np.asarray(ref, dtype=np.float64)
        return np.abs(y - ref) / np.spacing(np.abs(ref))

    x = np.concatenate([-rng.uniform(0, 700, 20000), -np.exp(rng.uniform(-40, 6, 20000)),
                        [-0.0, -700.0, -699.999, -5e-324, -1e-310, -1e-16]])
    y = eng.f64_math("exp", x)
    assert ulps(y, np.exp(x.astype(ld))).max() <= 2.0
    assert ulps(y, eng.f64_math("exp_lib", x)).max() <= 2.0
    edge = np.array([-700.5, -1000.0, -np.inf, np.nan, 0.0, 1.0, 3.5])
    np.testing.assert_array_equal(eng.f64_math("exp", edge), eng.f64_math("exp_lib", edge))

    x = np.concatenate([np.exp(rng.uniform(-700, 700, 20000)), -np.exp(rng.uniform(-700, 700, 5000)),
                        [1.0, 2.0, 3.0, 0.1, 1e-16]])
    y = eng.f64_math("rcp", x)
    assert ulps(y, ld(1) / x.astype(ld)).max() <= 1.0
    edge = np.array([0.0, -0.0, 1e-310, 5e-324, 1e308, -1e308, np.inf, np.nan])
    np.testing.assert_array_equal(eng.f64_math("rcp", edge), eng.f64_math("rcp_lib", edge))

    x = np.concatenate([np.exp(rng.uniform(-700, 700, 20000)), [1.0, 4.0, 2.0, 0.5, 9.869604401089358]])
    y = eng.f64_math("rsqrt", x)
    assert ulps(y, ld(1) / np.sqrt(x.astype(ld))).max() <= 2.0
    edge = np.array([0.0, 1e-310, 1e308, -1.0, np.inf, np.nan])
    np.testing.assert_array_equal(eng.f64_math("rsqrt", edge), eng.f64_math("rsqrt_lib", edge))


def test_ff_exp_log_accuracy(engine_factory):
    """Float-float e^x and ln x of the mixed solver's passes (tables of e^k, e^(j/256), ln c_j,
    1/c_j): within 2e-14 relative (ln x: of max(|ln x|, 1)) of long-double references at the
    float-pair value of x."""
    eng = engine_factory(12, 6)
    rng = np.random.default_rng(5)
    ld = np.longdouble

    def pair(x):
        h = x.astype(np.float32).astype(np.float64)
        return h + (x - h).astype(np.float32).astype(np.float64)

    # float-pair precision holds while the low part is a normal float: e^x >= 2^-102 (x >= -70)
    x = pair(np.concatenate([rng.uniform(-70.0, 87.9, 20000), rng.uniform(-1e-3, 1e-3, 2000),
                             [0.0, -0.5 / 256, 1.0 / 512, -70.0, 87.5]]))
    y = eng.f64_math("ff_exp", x)
    ref = np.exp(x.astype(ld))
    assert np.max(np.abs((y - ref) / ref)) <= 2e-14
    x = pair(rng.uniform(-87.0, -70.0, 2000))  # below: the resolution of the high part (subnormal at the end)
    y = eng.f64_math("ff_exp", x)
    ref = np.exp(x.astype(ld))
    assert np.max(np.abs((y - ref) / ref)) <= 1e-6
    x = pair(np.concatenate([np.exp(rng.uniform(-80, 80, 20000)), rng.uniform(0.99, 1.01, 2000),
                             [1.0, 2.0, 0.5, 1.00390625, 1.99999]]))
    y = eng.f64_math("ff_log", x)
    ref = np.log(x.astype(ld))
    assert np.max(np.abs(y - ref) / np.maximum(np.abs(ref), 1.0)) <= 2e-14


def test_thermo_matches_oracle(engine_factory, P):
    eng = engine_factory(64, 8)
    nd = orc.Nodes(64, 8)
    x, T, mu, xi = random_states(32, 11, mu_neg=True, asym=True)
    th = eng.thermo(x, T, mu, xi)
    for i in range(len(T)):
        ref = orc.thermo(P, nd, x[i], mu[i], T[i], xi[i])
        assert abs(th["pressure"][i] - ref["pressure"]) <= 1e-13 * abs(ref["pressure"])
        assert abs(th["entropy"][i] - ref["entropy"]) <= 1e-11 * max(1.0, abs(ref["entropy"]))
        assert abs(th["energy"][i] - ref["energy"]) <= 1e-11 * max(1.0, abs(ref["energy"]))
        np.testing.assert_allclose(th["rho"][i], ref["rho"], rtol=1e-11, atol=1e-13)
        np.testing.assert_allclose(th["n_q"][i], ref["nq"], rtol=1e-11, atol=1e-14)
        np.testing.assert_allclose(th["n_aq"][i], ref["naq"], rtol=1e-11, atol=1e-14)


def assert_solution_parity(res, i, ref, msg=""):
    assert bool(res["converged"][i]) == ref["converged"], (msg, i, res["status"][i], ref["status"])
    if not ref["converged"]:
        return
    x, xr = res["x"][i], ref["x"]
    assert np.all(np.abs(x[:3] - xr[:3]) <= 1e-9 * np.abs(xr[:3]) + 1e-12), (msg, i, x, xr)
    assert np.all(np.abs(x[3:] - xr[3:]) <= 1e-10), (msg, i, x, xr)
    assert abs(res["omega"][i] - ref["omega"]) <= 1e-12 * abs(ref["omega"]), (msg, i)
    assert abs(res["entropy"][i] - ref["entropy"]) <= 1e-9 * max(1.0, abs(ref["entropy"]))
    np.testing.assert_allclose(res["n_q"][i], ref["nq"], rtol=1e-9, atol=1e-12)


def test_multiseed_solve_matches_oracle(engine_factory, P):
    """The isotropic T x mu scan shape (xi = 0, p64/t8, MultiSeed) on a coarse 6 x 6 sub-grid."""
    eng = engine_factory(64, 8)
    nd = orc.Nodes(64, 8)
    Tg, mg = np.meshgrid(np.linspace(50, 300, 6), np.linspace(0, 400, 6), indexing="ij")
    T = Tg.ravel() / HBARC
    mu = mg.ravel() / HBARC
    table, hot = pnjl.multiseed_table()
    opts = SolveOptions(iterations=40)
    res = eng.solve(T, mu, 0.0, seed_table=table, seed_table_hot=hot, opts=opts)
    refs = orc.solve_batch(P, nd, T, np.repeat(mu[:, None], 3, 1), 0.0, multi=True, opts=orc.default_opts(max_iter=40))
    for i in range(T.size):
        ref = orc.result_to_dict(refs[i])
        assert_solution_parity(res, i, ref)
        assert res["chosen_seed"][i] == ref["chosen_seed"]
        assert res["iterations"][i] == ref["iterations"]
        assert res["status"][i] == ref["status"]


def test_anisotropic_asymmetric_solve_matches_oracle(engine_factory, P):
    """Anisotropic and flavour-asymmetric shapes: xi != 0, 4 seeds, mu_s = mu/2, p32/t8."""
    eng = engine_factory(32, 8)
    nd = orc.Nodes(32, 8)
    rng = np.random.default_rng(5)
    n = 24
    T = rng.uniform(20, 300, n) / HBARC
    mu1 = rng.uniform(0, 450, n) / HBARC
    mu = np.stack([mu1, mu1, 0.5 * mu1], axis=1)
    xi = rng.uniform(-0.4, 0.4, n)
    table, hot = pnjl.multiseed_table(4)
    res = eng.solve(T, mu, xi, seed_table=table, seed_table_hot=hot, opts=SolveOptions(iterations=40))
    refs = orc.solve_batch(P, nd, T, mu, xi, multi=True, n_seeds=4, opts=orc.default_opts(max_iter=40))
    for i in range(n):
        assert_solution_parity(res, i, orc.result_to_dict(refs[i]), "asym")


def test_per_point_seeds_and_multiseed_fallback(engine_factory, P):
    eng = engine_factory(24, 6)
    nd = orc.Nodes(24, 6)
    T = np.array([60.0, 100.0, 180.0, 250.0, 320.0]) / HBARC
    mu = np.array([340.0, 0.0, 200.0, 100.0, 10.0]) / HBARC
    seeds = np.array([pnjl.HADRON_SEED_5, pnjl.HIGH_DENSITY_SEED_5, (-3.0, -3.0, -3.0, 2.5, -1.0),
                      pnjl.QUARK_SEED_5, (-2.5, -0.1, -0.2, 0.9, 0.1)])
    table, hot = pnjl.multiseed_table()
    for fb in (True, False):
        opts = SolveOptions(iterations=40, auto_multiseed_fallback=fb)
        res = eng.solve(T, mu, 0.0, seed_table=table, seed_table_hot=hot, point_seeds=seeds, opts=opts)
        for i in range(T.size):
            ref = orc.solve_point(P, nd, T[i], [mu[i]] * 3, 0.0, seeds[i], False,
                                  orc.default_opts(max_iter=40, auto_multiseed_fallback=int(fb)))
            assert_solution_parity(res, i, ref, f"fallback={fb}")
            assert res["status"][i] == ref["status"], (i, fb)
            assert res["iterations"][i] == ref["iterations"], (i, fb)


def test_golden_scan_through_gpu(engine_factory):
    """The reference's stored scan (xi = 0, p12/t6) reproduced through the GPU solver."""
    from julia_relaxtime_gb300.scan import ScanOptions, gpu_point_solver, scan_rows
    from test_oracle_golden import check_scan_rows

    eng = engine_factory(12, 6)
    for fname, xis, exact in (("gap_transport_scan_xi0.csv", [0.0], True),
                              ("gap_transport_scan_xim0p6to0p6.csv", [-0.6, -0.4, -0.2, 0.0, 0.2, 0.4, 0.6], False)):
        g = read_csv(fname)
        gk = {(float(r["T_MeV"]), float(r["muB_MeV"]), float(r["xi"])): r for r in g}
        opts = ScanOptions(xi_values=xis, tmin_mev=120, tmax_mev=400, tstep_mev=10, mubmin_mev=0, mubmax_mev=800,
                           mubstep_mev=800, p_num=12, t_num=6, max_iter=40,
                           boundary_path=os.path.join(GOLDEN, "boundary.csv"), cep_path=os.path.join(GOLDEN, "cep.csv"))
        rows = scan_rows(opts, gpu_point_solver(12, 6, engine=eng))
        mism = check_scan_rows(rows, gk, exact_iterations=exact)
        assert mism <= 10
        # every row carries build_K_data of its solution (run_gap_transport_scan.jl:436-438)
        T = np.array([r["T_fm"] for r in rows])
        mq = np.array([r["muq_fm"] for r in rows])
        masses = np.array([[r["m_u"], r["m_d"], r["m_s"]] for r in rows])
        x = np.array([[0.0, 0.0, 0.0, r["Phi"], r["Phibar"]] for r in rows])
        ref = orc.kdata(orc.default_params(), T, mq, mq, masses, x)
        for k, v in ref.items():
            got = np.array([r["kdata"][k] for r in rows])
            assert np.all(np.abs(got - v) <= 1e-13 * np.abs(v).max()), k


def test_edge_cases(engine_factory, P):
    eng = engine_factory(16, 4)
    table, hot = pnjl.multiseed_table()
    opts = SolveOptions(iterations=40)
    # empty batch
    r0 = eng.solve(np.zeros(0), np.zeros(0), np.zeros(0), seed_table=table, opts=opts)
    assert r0["x"].shape == (0, 5)
    # invalid inputs are flagged per point, valid neighbours still solve
    T = np.array([0.0, -0.5, np.nan, 0.5, 0.5, 0.5]) / 1.0
    mu = np.array([0.5, 0.5, 0.5, np.inf, 0.5, 0.5])
    xi = np.array([0.0, 0.0, 0.0, 0.0, -1.0, 0.1])
    r = eng.solve(T, mu, xi, seed_table=table, seed_table_hot=hot, opts=opts)
    assert list(r["status"][:5]) == [api.PNJL_POINT_INVALID_INPUT] * 5
    assert r["status"][5] == api.PNJL_POINT_CONVERGED and r["converged"][5]
    # a non-finite seed raises inside the reference's nlsolve: status EXCEPTION, no fallback
    seeds = np.array([[np.nan, -1.0, -2.0, 0.1, 0.1]])
    r = eng.solve(np.array([0.5]), np.array([0.5]), 0.0, seed_table=table, seed_table_hot=hot, point_seeds=seeds,
                  opts=opts)
    assert r["status"][0] == api.PNJL_POINT_EXCEPTION and not r["converged"][0]
    # iteration cap: max_iter = 1 gives the oracle's (unconverged) outcome
    nd = orc.Nodes(16, 4)
    r = eng.solve(np.array([0.5]), np.array([1.5]), 0.0, seed_table=table, seed_table_hot=hot,
                  opts=SolveOptions(iterations=1, trust_region_fallback=False))
    ref = orc.solve_point(P, nd, 0.5, [1.5] * 3, 0.0, orc.multiseed_seeds(P, 0.5), True,
                          orc.default_opts(max_iter=1, trust_region_fallback=0))
    assert r["status"][0] == ref["status"] and bool(r["converged"][0]) == ref["converged"]
    # bad options are rejected with an error code and message
    with pytest.raises(api.CudaLibraryError, match="seed table"):
        eng.solve(np.array([0.5]), np.array([0.5]), 0.0, seed_table=np.zeros((0, 5)), opts=opts)
    with pytest.raises(api.CudaLibraryError, match="node counts"):
        eng.set_nodes(0, 4)


def test_solve_api_mirrors_reference(engine_factory):
    eng = engine_factory(24, 6)
    T, mu = 100 / HBARC, 200 / HBARC
    r = pnjl.solve(pnjl.FixedMu(), T, mu, p_num=24, t_num=6, engine=eng)
    assert r.converged and r.iterations > 0
    assert r.pressure == pytest.approx(-r.omega, rel=1e-12)          # test_solver_implicit.jl:56-59
    assert r.masses[0] == pytest.approx(r.masses[1], rel=1e-6)       # :233-240
    assert r.masses[2] > r.masses[0]
    r2 = pnjl.solve(pnjl.FixedMu(), T, mu, xi=0.2, p_num=24, t_num=6, engine=eng)
    assert r2.converged and r2.xi == 0.2
    rm = pnjl.solve(pnjl.FixedMu(), T, mu, seed_strategy=pnjl.MultiSeed(), p_num=24, t_num=6, engine=eng)
    assert rm.converged and abs(rm.omega - r.omega) < 1e-10
    # the two regression points of test_solver_random_physical_smoke.jl:33-51 (p12/t4)
    for T_MeV, muB, xi in ((48.269077, 972.6409, 0.479315), (288.453662, 563.275131, -0.652469)):
        rr = pnjl.solve(pnjl.FixedMu(), T_MeV / HBARC, muB / 3 / HBARC, xi=xi, p_num=12, t_num=4, engine=eng)
        assert rr.converged
        assert -1e-8 <= rr.x_state[3] <= 1 + 1e-8 and np.all(rr.masses > 0)


@pytest.mark.parametrize("p_num,t_num,asym", [(64, 8, False), (32, 8, True)])
def test_mixed_precision_matches_fp64_oracle(engine_factory, P, p_num, t_num, asym):
    """PNJL_PREC_MIXED: FP32 Kahan-compensated Newton passes, FP64 refinement and certification.
    The certified roots and the selected phase must match the FP64 oracle (required bound
    |dphi|/|phi| <= 1e-9, |dPhi| <= 1e-10; Omega 1e-12 relative); iteration counts differ by
    construction and are not compared."""
    eng = engine_factory(p_num, t_num)
    nd = orc.Nodes(p_num, t_num)
    rng = np.random.default_rng(23 + p_num)
    n = 40
    T = rng.uniform(40, 320, n) / HBARC
    mu1 = rng.uniform(0, 420, n) / HBARC
    mu = np.stack([mu1, mu1, (0.5 if asym else 1.0) * mu1], axis=1)
    xi = rng.uniform(-0.5, 0.5, n) if asym else np.zeros(n)
    ns = 4 if asym else 6
    table, hot = pnjl.multiseed_table(ns)
    ftol = 1e-11
    res = eng.solve(T, mu, xi, seed_table=table, seed_table_hot=hot,
                    opts=SolveOptions(iterations=40, ftol=ftol, precision="mixed"))
    refs = orc.solve_batch(P, nd, T, mu, xi, multi=True, n_seeds=ns, opts=orc.default_opts(max_iter=40, ftol=ftol))
    st = eng.stats()
    assert st["passes_fp32"] > 0 and st["node_evals_fp32"] > 0
    for i in range(n):
        ref = orc.result_to_dict(refs[i])
        assert bool(res["converged"][i]) == ref["converged"], (i, res["status"][i], ref["status"])
        if not ref["converged"]:
            continue
        assert res["residual_norm"][i] < ftol
        x, xr = res["x"][i], ref["x"]
        assert np.all(np.abs(x[:3] - xr[:3]) <= 1e-9 * np.abs(xr[:3]) + 1e-12), (i, x, xr)
        assert np.all(np.abs(x[3:] - xr[3:]) <= 1e-10), (i, x, xr)
        assert abs(res["omega"][i] - ref["omega"]) <= 1e-12 * abs(ref["omega"]), i
        np.testing.assert_allclose(res["n_q"][i], ref["nq"], rtol=1e-9, atol=1e-12)


def test_mixed_per_point_seed_and_fallback(engine_factory, P):
    eng = engine_factory(24, 6)
    nd = orc.Nodes(24, 6)
    T = np.array([60.0, 100.0, 180.0, 250.0, 320.0]) / HBARC
    mu = np.array([340.0, 0.0, 200.0, 100.0, 10.0]) / HBARC
    seeds = np.array([pnjl.HADRON_SEED_5, pnjl.HIGH_DENSITY_SEED_5, (-3.0, -3.0, -3.0, 2.5, -1.0),
                      pnjl.QUARK_SEED_5, (-2.5, -0.1, -0.2, 0.9, 0.1)])
    table, hot = pnjl.multiseed_table()
    res = eng.solve(T, mu, 0.0, seed_table=table, seed_table_hot=hot, point_seeds=seeds,
                    opts=SolveOptions(iterations=40, ftol=1e-11, precision="mixed"))
    for i in range(T.size):
        ref = orc.solve_point(P, nd, T[i], [mu[i]] * 3, 0.0, seeds[i], False,
                              orc.default_opts(max_iter=40, ftol=1e-11))
        assert bool(res["converged"][i]) == ref["converged"], i
        if ref["converged"]:
            assert abs(res["omega"][i] - ref["omega"]) <= 1e-12 * abs(ref["omega"]), i
            assert np.all(np.abs(res["x"][i][3:] - ref["x"][3:]) <= 1e-10), i


def test_tmu_scan_gpu_matches_oracle(engine_factory):
    """run_tmu_scan (TmuScan.jl:120-234) through the GPU point solver: the same rows, branches,
    candidate messages and iteration counts as the same driver over the oracle."""
    import os

    from julia_relaxtime_gb300 import scan
    from oracle_adapter import GOLDEN, oracle_point_solver

    eng = engine_factory(24, 8)
    kw = dict(boundary_path=os.path.join(GOLDEN, "boundary.csv"), cep_path=os.path.join(GOLDEN, "cep.csv"))
    Ts, mus = [50.0, 130.0, 200.0], np.arange(0.0, 401.0, 10.0)
    rows_g, st_g = scan.tmu_scan_rows(Ts, mus, [0.0, 0.2], scan.gpu_point_solver(24, 8, engine=eng), **kw)
    rows_o, st_o = scan.tmu_scan_rows(Ts, mus, [0.0, 0.2], oracle_point_solver(24, 8), **kw)
    assert st_g == st_o
    for (T, mu, xi, r, msg), (T2, mu2, xi2, r2, msg2) in zip(rows_g, rows_o):
        assert (T, mu, xi) == (T2, mu2, xi2)
        assert msg == msg2
        assert r["converged"] == r2["converged"] and r["iterations"] == r2["iterations"], (T, mu, xi)
        np.testing.assert_allclose(r["x"], r2["x"], rtol=1e-9, atol=1e-11)
        assert r["pressure"] == pytest.approx(r2["pressure"], rel=1e-12, abs=1e-13)
        a = [float(v) for v in scan.format_tmu_row(T, mu, xi, r, msg).split(",")[:15]]
        b = [float(v) for v in scan.format_tmu_row(T2, mu2, xi2, r2, msg2).split(",")[:15]]
        assert np.allclose(a, b, rtol=0, atol=1.01e-6), (a, b)  # 6-decimal columns, last digit


def test_mixed_pipeline_chunks_and_autotune(engine_factory):
    """The launch forms of mixed per-point solves (one fused kernel, with 0, 1 or 3
    certifying warps per block; the per-point and task kernels one after the other; the
    two-stream chunk pipeline) and the autotuner change launch shapes only: bit-identical
    results for every shape."""
    import torch

    eng = engine_factory(32, 8)
    rng = np.random.default_rng(77)
    n = 3000
    T = rng.uniform(50, 300, n) / HBARC
    mu = rng.uniform(0, 400, n) / HBARC
    xi = rng.uniform(-0.4, 0.4, n)
    seeds = np.where((T * HBARC < 160)[:, None], np.array(pnjl.HADRON_SEED_5), np.array(pnjl.QUARK_SEED_5))
    table, hot = pnjl.multiseed_table(4)
    opts = SolveOptions(iterations=40, ftol=1e-10, precision="mixed", verify_seeds=-1, verify_T_max_MeV=170.0,
                        verify_max_step=0.3)
    outs = []
    for chunks, cert in ((1, 0), (1, 1), (1, 3), (-1, 0), (3, 0), (7, 0)):
        eng.set_tuning(32, 0, pipeline_chunks=chunks, cert_warps=cert)
        outs.append(eng.solve(T, mu, xi, seed_table=table, seed_table_hot=hot, point_seeds=seeds, opts=opts))
        st = eng.stats()
        assert st["kernel_launches"] > 0 and st["device_wait_timeouts"] == 0
    for r in outs[1:]:
        for k in ("x", "omega", "entropy", "n_q", "status", "chosen_seed", "iterations", "converged"):
            np.testing.assert_array_equal(r[k], outs[0][k], err_msg=k)
    assert outs[0]["converged"].mean() > 0.99
    # autotuner over the table-mode mixed solve of the same points (device arrays)
    dev = torch.device("cuda", 0)
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in (("T", T), ("mu", mu), ("xi", xi))}
    d_out = {"x": torch.empty(5 * n, dtype=torch.float64, device=dev),
             "omega": torch.empty(n, dtype=torch.float64, device=dev),
             "converged": torch.empty(n, dtype=torch.uint8, device=dev)}
    torch.cuda.synchronize()
    m = d["mu"].data_ptr()
    best, tried = eng.autotune(n, d["T"].data_ptr(), m, m, m, d["xi"].data_ptr(),
                               {k: v.data_ptr() for k, v in d_out.items()}, seed_table=table, seed_table_hot=hot,
                               opts=SolveOptions(iterations=40, ftol=1e-10, precision="mixed"), reps=1)
    assert len(tried) >= 1 and best["ms"] == min(t["ms"] for t in tried) and best["ms"] > 0
    tu = eng.tuning()
    assert tu["blocks_per_sm"] == best["blocks_per_sm"] and tu["pipeline_chunks"] == best["pipeline_chunks"]
    ref = eng.solve(T, mu, xi, seed_table=table, seed_table_hot=hot,
                    opts=SolveOptions(iterations=40, ftol=1e-10, precision="mixed"))
    np.testing.assert_array_equal(d_out["omega"].cpu().numpy(), ref["omega"])
    eng.set_tuning(32, 0, pipeline_chunks=0, cert_warps=0)


def test_mixed_table_mode_independent_of_timing(engine_factory):
    """MultiSeed table mode (all seeds of a point as concurrent tasks, duplicate roots of
    earlier seeds skipped or waited for): the same results, bit for bit, over repeated
    launches and launch shapes, so the order in which seeds finish never shows."""
    eng = engine_factory(32, 8)
    rng = np.random.default_rng(91)
    n = 2500
    T = rng.uniform(50, 300, n) / HBARC
    mu = rng.uniform(0, 400, n) / HBARC
    xi = rng.uniform(-0.4, 0.4, n)
    table, hot = pnjl.multiseed_table(6)
    opts = SolveOptions(iterations=40, ftol=1e-10, precision="mixed")
    outs = []
    for bps in (1, 2, 1, 2):
        eng.set_tuning(32, bps, pipeline_chunks=0, cert_warps=0)
        outs.append(eng.solve(T, mu, xi, seed_table=table, seed_table_hot=hot, opts=opts))
        assert eng.stats()["device_wait_timeouts"] == 0
    for r in outs[1:]:
        for k in ("x", "omega", "entropy", "status", "chosen_seed", "iterations", "converged"):
            np.testing.assert_array_equal(r[k], outs[0][k], err_msg=k)
    assert outs[0]["converged"].mean() > 0.99
    eng.set_tuning(32, 0, pipeline_chunks=0, cert_warps=0)


def test_plan_mixed_orders_one_graph(engine_factory):
    """Mixed quadrature orders: the same T x mu grid at p = 64, 128 and 256 momentum nodes (plus an FP64
    per-point segment and a learned-seed segment) captured into one CUDA graph and replayed:
    every segment equals the same solve launched on its own, on every replay."""
    import torch

    from julia_relaxtime_gb300.engine import SolvePlan
    from julia_relaxtime_gb300.learned_seed import LearnedSeed

    eng = engine_factory(64, 8)
    dev = torch.device("cuda", 0)
    Tg, mg = np.meshgrid(np.linspace(50, 300, 12), np.linspace(0, 400, 12), indexing="ij")
    T = Tg.ravel() / HBARC
    mu = mg.ravel() / HBARC
    n = T.size
    xi = np.zeros(n)
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in (("T", T), ("mu", mu), ("xi", xi))}
    table, hot = pnjl.multiseed_table(6)
    seeds = np.tile(np.array(pnjl.HADRON_SEED_5), (n, 1))
    d_seeds = torch.from_numpy(seeds.ravel().copy()).to(dev)
    ls = LearnedSeed(eng, seed=5)
    ls.default_scaling(np.tile(np.array(pnjl.HADRON_SEED_5), (4, 1)) + np.arange(4)[:, None] * 0.1)
    mixed = SolveOptions(iterations=40, ftol=1e-10, precision="mixed")
    fp64 = SolveOptions(iterations=40, ftol=1e-10, precision="fp64")
    segs = [(64, mixed, 0, False), (128, mixed, 0, False), (256, mixed, 0, False),
            (32, fp64, d_seeds.data_ptr(), False), (64, mixed, 0, True)]

    def outputs():
        return {"x": torch.empty(5 * n, dtype=torch.float64, device=dev),
                "omega": torch.empty(n, dtype=torch.float64, device=dev),
                "status": torch.empty(n, dtype=torch.int32, device=dev),
                "converged": torch.empty(n, dtype=torch.uint8, device=dev)}

    m = d["mu"].data_ptr()
    plan = SolvePlan(eng)
    outs = []
    for p_num, o, ps, learned in segs:
        out = outputs()
        outs.append(out)
        plan.add(p_num, 8, n, d["T"].data_ptr(), m, m, m, d["xi"].data_ptr(), {k: v.data_ptr() for k, v in out.items()},
                 seed_table=table, seed_table_hot=hot, opts=o, learned=learned, d_point_seeds=ps)
    torch.cuda.synchronize()
    plan.finalize()
    first = None
    for rep in range(2):
        for out in outs:
            out["omega"].fill_(0.0)
        plan.launch()
        eng.synchronize()
        got = [{k: v.cpu().numpy().copy() for k, v in out.items()} for out in outs]
        if first is None:
            first = got
        else:
            for a, b in zip(got, first):
                for k in a:
                    np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    st = plan.stats()
    assert st["points"] == 5 * n and st["kernel_launches"] >= 5 and st["last_kernel_ms"] > 0
    # each segment alone, through the context with its own node tables
    for (p_num, o, ps, learned), g in zip(segs, first):
        eng.set_nodes(p_num, 8)
        ref = outputs()
        eng.solve_device(n, d["T"].data_ptr(), m, m, m, d["xi"].data_ptr(), {k: v.data_ptr() for k, v in ref.items()},
                         seed_table=table, seed_table_hot=hot, opts=o, learned=learned, d_point_seeds=ps)
        eng.synchronize()
        for k, v in ref.items():
            np.testing.assert_array_equal(v.cpu().numpy(), g[k], err_msg=f"p{p_num} {k}")
        assert g["converged"].mean() > 0.95
    # higher orders move the solution by the quadrature error only
    d64, d256 = first[0]["x"].reshape(n, 5), first[2]["x"].reshape(n, 5)
    both = first[0]["converged"].astype(bool) & first[2]["converged"].astype(bool)
    assert np.median(np.abs(d64[both] - d256[both])) < 1e-2
    plan.close()


def test_unstable_branch_root_gets_verified(engine_factory):
    """A per-point seed that converges to the unstable branch between two coexisting phases
    (T = 136.35 MeV, mu_u = mu_d = 250 MeV, mu_s = 125 MeV, xi = -0.4; three roots) is
    verified by the MultiSeed candidates although the point lies outside the verification
    region and the root is close to the seed: the result is the min-Omega root of the plain
    multi-seed solve, in mixed precision and in FP64."""
    eng = engine_factory(128, 32)
    T = np.array([136.3458720078163]) / HBARC
    mu = np.array([[250.0, 250.0, 125.0]]) / HBARC
    xi = np.array([-0.4])
    seed = np.array([[-1.1634, -1.1634, -2.111, 0.2479, 0.2862]])  # the learned seed there
    table, hot = pnjl.multiseed_table(6, (pnjl.MEDIUM_SEED_5, pnjl.HIGH_DENSITY_SEED_5))
    ref = eng.solve(T, mu, xi, seed_table=table, seed_table_hot=hot,
                    opts=SolveOptions(iterations=40, ftol=1e-10, precision="fp64"))
    assert ref["converged"][0]
    for precision, cert in (("mixed", 0), ("mixed", 2), ("fp64", 0)):
        eng.set_tuning(32, 0, pipeline_chunks=0, cert_warps=cert)  # 2: certification deferred to other warps
        base = dict(iterations=40, ftol=1e-10, precision=precision, verify_T_max_MeV=0.0, verify_max_step=10.0)
        alone = eng.solve(T, mu, xi, seed_table=table, seed_table_hot=hot, point_seeds=seed,
                          opts=SolveOptions(verify_seeds=0, **base))
        assert alone["converged"][0] and alone["omega"][0] > ref["omega"][0] + 1e-3  # the unstable branch
        r = eng.solve(T, mu, xi, seed_table=table, seed_table_hot=hot, point_seeds=seed,
                      opts=SolveOptions(verify_seeds=-1, **base))
        assert r["converged"][0] and r["residual_norm"][0] <= 1e-10
        assert abs(r["omega"][0] - ref["omega"][0]) <= 1e-10 * abs(ref["omega"][0]), precision
        np.testing.assert_allclose(r["x"][0], ref["x"][0], rtol=1e-8, atol=1e-10)
    eng.set_tuning(32, 0, pipeline_chunks=0, cert_warps=0)
