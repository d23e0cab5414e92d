"""The dual-branch scan and phase-boundary driver (julia_relaxtime_gb300.phase) on the CPU
oracle: the reference's stored dual_branch_T50.csv (run_dual_branch_scan(T_mev=50,
mu_range=0:5:400) + merge_branches, p24/t8) is reproduced row by row, and the transition it
implies lies on the reference's first-order line (data/reference/pnjl/boundary.csv)."""
import os

import numpy as np
import pytest

from julia_relaxtime_gb300 import phase
from oracle import oracle as orc
from oracle_adapter import GOLDEN, read_csv, results_to_arrays


def oracle_branch_solver(p_num=24, t_num=8):
    P = orc.default_params()
    nd = orc.Nodes(p_num, t_num)

    def solver(T, mu, xi, seeds):
        mu3 = np.repeat(np.asarray(mu, dtype=np.float64).reshape(-1, 1), 3, axis=1)
        rs = orc.solve_batch(P, nd, T, mu3, xi, seeds=seeds, multi=False, opts=orc.default_opts())
        return results_to_arrays(rs)

    return solver


@pytest.fixture(scope="module")
def t50():
    return phase.run_dual_branch_scan(50.0, np.arange(0.0, 400.001, 5.0), 0.0, solver=oracle_branch_solver())


def test_dual_branch_T50_reproduces_reference_csv(t50, tmp_path):
    out = tmp_path / "dual_branch_T50.csv"
    rows = phase.merge_branches(t50, output_path=str(out))
    gold = read_csv("dual_branch_T50.csv")
    assert len(rows) == len(gold)
    with open(out) as fh:
        header = fh.readline().strip().split(",")
    assert header == phase.MERGED_HEADER
    for r, g in zip(rows, gold):
        assert r["mu_MeV"] == float(g["mu_MeV"]) and r["branch"] == g["branch"], (r["mu_MeV"], r["branch"], g["branch"])
        for k in ("omega", "pressure", "rho", "phi_u", "phi_s", "Phi1", "Phi2"):
            assert abs(r[k] - float(g[k])) < 2e-9, (r["mu_MeV"], k, r[k], g[k])
        for k in ("M_u_MeV", "M_s_MeV"):
            assert abs(r[k] - float(g[k])) < 2e-6, (r["mu_MeV"], k)
        if g["delta_omega"] == "NaN":
            assert np.isnan(r["delta_omega"])
        else:
            assert abs(r["delta_omega"] - float(g["delta_omega"])) < 2e-9


def test_transition_on_reference_first_order_line(t50):
    info = phase.find_phase_transition(t50)
    assert info.found
    assert info.mu_quark_spinodal < info.mu_c < info.mu_hadron_spinodal
    lo, hi = info.coexistence_region
    assert lo <= info.mu_c <= hi
    gold = [r for r in read_csv("boundary.csv") if float(r["xi"]) == 0.0 and float(r["T_MeV"]) == 50.0][0]
    # the reference's line comes from T-rho scans with a Maxwell construction at its own nodes;
    # the Omega crossing of the two branches on a 5 MeV mu grid lands within 1 MeV of it
    assert abs(info.mu_c - float(gold["mu_transition_MeV"])) < 1.0, (info.mu_c, gold["mu_transition_MeV"])


def test_boundary_and_cep_writers(tmp_path):
    rows = [dict(xi=0.0, T_MeV=50.0, mu_transition_MeV=356.4, rho_hadron=0.08, rho_quark=2.59)]
    phase.write_boundary_csv(rows, str(tmp_path / "b.csv"))
    phase.write_cep_csv([dict(xi=0.2, T_CEP_MeV=123.0, mu_CEP_MeV=316.06)], str(tmp_path / "c.csv"))
    from julia_relaxtime_gb300.pnjl import load_phase_boundary

    data = load_phase_boundary(0.0, str(tmp_path / "b.csv"), os.path.join(GOLDEN, "cep.csv"))
    assert data.T_values.size == 1 and data.mu_values[0] == 356.4
    assert (tmp_path / "c.csv").read_text().startswith("xi,T_CEP_MeV,mu_CEP_MeV\n0.2,123.0,316.06")


@pytest.mark.gpu
def test_dual_branch_and_boundary_through_gpu(engine_factory, t50):
    """The same scans through the GPU solver (batched lines): the T = 50 MeV rows of the
    reference file, the first-order line of boundary.csv at xi = 0, 0.2, 0.4 (mu_c within
    0.05 MeV, rho of both branches within 0.01 rho0), and the CEP of cep.csv."""
    eng = engine_factory(24, 8)
    solver = phase.gpu_branch_solver(24, 8, engine=eng)
    g = phase.run_dual_branch_scan(50.0, np.arange(0.0, 400.001, 5.0), 0.0, solver=solver)
    rows_g = phase.merge_branches(g)
    rows_o = phase.merge_branches(t50)
    assert [r["branch"] for r in rows_g] == [r["branch"] for r in rows_o]
    for a, b in zip(rows_g, rows_o):
        assert abs(a["omega"] - b["omega"]) < 1e-11 and abs(a["phi_u"] - b["phi_u"]) < 1e-9
    gold = {(float(r["xi"]), float(r["T_MeV"])): r for r in read_csv("boundary.csv")}
    rows = phase.phase_boundary([0.0, 0.2, 0.4], [50.0, 80.0, 100.0], np.arange(200.0, 450.001, 5.0), solver=solver)
    assert len(rows) == 9
    for r in rows:
        ref = gold[(r["xi"], r["T_MeV"])]
        assert abs(r["mu_transition_MeV"] - float(ref["mu_transition_MeV"])) < 0.05, (r, ref)
        assert abs(r["rho_hadron"] - float(ref["rho_hadron"])) < 0.01 and abs(r["rho_quark"] - float(ref["rho_quark"])) < 0.01
    cep = phase.locate_cep([0.0, 0.2, 0.4], np.arange(200.0, 450.001, 5.0), 90.0, 150.0, tol_mev=0.1, solver=solver)
    gold_cep = {float(r["xi"]): r for r in read_csv("cep.csv")}
    for c in cep:
        ref = gold_cep[c["xi"]]
        assert abs(c["T_CEP_MeV"] - float(ref["T_CEP_MeV"])) < 1.5, (c, ref)
        assert abs(c["mu_CEP_MeV"] - float(ref["mu_CEP_MeV"])) < 4.0, (c, ref)
