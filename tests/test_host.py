"""Host-side logic of the package (no GPU): seed strategies, phase boundary, scan grid,
CSV formatting and resume keys, parameter loading, C-ABI declarations."""
import math
import os

import numpy as np
import pytest

from julia_relaxtime_gb300 import pnjl
from julia_relaxtime_gb300.constants import PNJLParams, load_pnjl_config
from julia_relaxtime_gb300.scan import HEADER, ScanOptions, format_row, julia_range, julia_string, read_existing_keys
from oracle import oracle as orc
from oracle_adapter import GOLDEN, read_csv

HBARC = 197.327


def test_params_match_reference_constants():
    p = PNJLParams.default()
    o = orc.default_params()
    for k, _ in orc.Params._fields_:
        assert getattr(p, k) == pytest.approx(getattr(o, k), rel=1e-15)
    assert p.Lambda == pytest.approx(602.3 / 197.327)
    assert p.G * p.Lambda ** 2 == pytest.approx(1.835)


def test_load_pnjl_config_profiles(tmp_path):
    (tmp_path / "stiff.toml").write_text("[model]\nLambda_MeV = 631.4\n")
    cfg = load_pnjl_config("stiff", str(tmp_path))
    assert cfg["config"]["model"]["Lambda_MeV"] == 631.4
    assert cfg["config"]["model"]["G_over_Lambda2"] == 1.835  # deep merge keeps the rest
    p = PNJLParams.from_config(cfg["config"])
    assert p.Lambda == pytest.approx(631.4 / 197.327)
    with pytest.warns(UserWarning):
        load_pnjl_config("missing", str(tmp_path))


def test_multiseed_table_matches_reference_seeds():
    P = orc.default_params()
    cold, hot = pnjl.multiseed_table()
    np.testing.assert_array_equal(cold, orc.multiseed_seeds(P, 100 / HBARC))
    np.testing.assert_array_equal(hot, orc.multiseed_seeds(P, 300 / HBARC))
    assert np.array_equal(orc.builtin_seed("HADRON"), np.array(pnjl.HADRON_SEED_5))
    assert np.array_equal(orc.builtin_seed("HIGH_DENSITY"), np.array(pnjl.HIGH_DENSITY_SEED_5))


def test_default_seed_rules():
    mode = pnjl.FixedMu()
    s = pnjl.DefaultSeed()
    assert tuple(s.get_seed([100 / HBARC, 100 / HBARC], mode)) == pnjl.HADRON_SEED_5
    assert tuple(s.get_seed([160 / HBARC, 0.0], mode)) == pnjl.QUARK_SEED_5
    assert tuple(s.get_seed([100 / HBARC, 310 / HBARC], mode)) == pnjl.QUARK_SEED_5
    assert tuple(s.get_seed([300 / HBARC * (1 + 1e-12), 0.0], mode)) == pnjl.VERY_HIGH_TEMP_SEED_5
    assert pnjl.auto_phase_hint(150 / HBARC, 300 / HBARC) == "hadron"


def test_default_omega_selector_first_minimum():
    R = pnjl.SolverResult
    mk = lambda om, c: R(pnjl.FixedMu(), c, None, None, None, om, -om, 0, 0, 0, None, 1, 0.0, 0.0)  # noqa: E731
    rs = [mk(-1.0, False), mk(-2.0, True), mk(-3.0, True), mk(-3.0, True)]
    assert pnjl.default_omega_selector(rs) is rs[2]
    assert pnjl.default_omega_selector([mk(1.0, False)]).omega == 1.0


def test_phase_boundary_and_interpolation():
    b = os.path.join(GOLDEN, "boundary.csv")
    c = os.path.join(GOLDEN, "cep.csv")
    d = pnjl.load_phase_boundary(0.0, b, c)
    assert d.T_CEP == pytest.approx(130.9423828125)
    assert np.all(np.diff(d.T_values) > 0)
    assert pnjl.interpolate_mu_c(d, 140.0) != pnjl.interpolate_mu_c(d, 140.0)  # NaN above T_CEP
    assert pnjl.interpolate_mu_c(d, 10.0) == d.mu_values[0]  # clamped below the table
    T0, T1 = d.T_values[0], d.T_values[1]
    mid = pnjl.interpolate_mu_c(d, 0.5 * (T0 + T1))
    assert mid == pytest.approx(0.5 * (d.mu_values[0] + d.mu_values[1]))
    # xi without data -> no boundary -> plain continuation
    e = pnjl.load_phase_boundary(0.3, b, c)
    assert e.T_values.size == 0 and math.isnan(e.T_CEP)


def test_phase_aware_continuity_seed_switches_on_crossing():
    b = os.path.join(GOLDEN, "boundary.csv")
    c = os.path.join(GOLDEN, "cep.csv")
    s = pnjl.PhaseAwareContinuitySeed(0.0, boundary_path=b, cep_path=c)
    mode = pnjl.FixedMu()
    T = 80.0
    muc = pnjl.interpolate_mu_c(s.boundary_data, T)
    # first point: default seed of the current phase
    assert tuple(s.get_seed([T / HBARC, (muc - 20) / HBARC], mode)) == pnjl.HADRON_SEED_5
    assert tuple(s.get_seed([T / HBARC, (muc + 20) / HBARC], mode)) == pnjl.QUARK_SEED_5
    prev = np.array([-1.7, -1.7, -2.2, 0.01, 0.02])
    s.update(prev, T, muc - 20)
    assert s.previous_phase == "hadron"
    np.testing.assert_array_equal(s.get_seed([T / HBARC, (muc - 10) / HBARC], mode), prev)   # same phase
    assert tuple(s.get_seed([T / HBARC, (muc + 10) / HBARC], mode)) == pnjl.QUARK_SEED_5  # crossed
    s.update(prev, 150.0, 100.0)
    assert s.previous_phase == "crossover"
    np.testing.assert_array_equal(s.get_seed([T / HBARC, (muc + 10) / HBARC], mode), prev)
    s.reset()
    assert s.previous_solution is None and s.previous_phase == "unknown"
    s.set_phase("quark")
    assert s.previous_phase == "quark"
    # without boundary data: plain continuation after the first point
    s2 = pnjl.PhaseAwareContinuitySeed()
    assert tuple(s2.get_seed([200 / HBARC, 0.0], mode)) == pnjl.QUARK_SEED_5
    s2.update(prev)
    np.testing.assert_array_equal(s2.get_seed([10 / HBARC, 0.0], mode), prev)


def test_continuity_seed():
    s = pnjl.ContinuitySeed()
    mode = pnjl.FixedMu()
    assert tuple(s.get_seed([0.2, 0.1], mode)) == pnjl.HADRON_SEED_5
    s.update([1, 2, 3, 4, 5])
    assert list(s.get_seed([0.2, 0.1], mode)) == [1, 2, 3, 4, 5]
    s.reset()
    assert s.previous_solution is None


@pytest.mark.parametrize("fname", ["gap_transport_scan_xi0.csv", "gap_transport_scan_xim0p6to0p6.csv"])
def test_julia_string_roundtrips_reference_text(fname):
    with open(os.path.join(GOLDEN, fname)) as fh:
        header = fh.readline().strip().split(",")
        n = 0
        for line in fh:
            for k, v in zip(header, line.strip().split(",")):
                if k in ("converged", "iterations"):
                    continue
                assert julia_string(float(v)) == v, (k, v, julia_string(float(v)))
                n += 1
    assert n > 1000


def test_julia_string_edge_cases():
    assert julia_string(1e-5) == "1.0e-5"
    assert julia_string(0.0001) == "0.0001"
    assert julia_string(123456.0) == "123456.0"
    assert julia_string(1e6) == "1.0e6"
    assert julia_string(-0.0) == "-0.0"
    assert julia_string(float("nan")) == "NaN"
    assert julia_string(float("-inf")) == "-Inf"
    assert julia_string(2.5e-300) == "2.5e-300"


def test_scan_grid_and_rows_shape(tmp_path):
    assert julia_range(50.0, 200.0, 10.0)[-1] == 200.0 and len(julia_range(50.0, 200.0, 10.0)) == 16
    assert len(julia_range(0.0, 1200.0, 60.0)) == 21
    # the 47 columns of run_gap_transport_scan.jl:274-291; the golden files keep a subset in order
    assert len(HEADER) == 47
    with open(os.path.join(GOLDEN, "gap_transport_scan_xi0.csv")) as fh:
        gcols = fh.readline().strip().split(",")
    assert [c for c in HEADER if c in gcols] == gcols
    row = {k: float("nan") for k in HEADER}
    row.update(converged=True, iterations=3, T_MeV=120.0)
    text = format_row(row)
    assert text.count(",") == 46 and text.startswith("120.0,NaN")


def test_resume_keys(tmp_path):
    p = tmp_path / "scan.csv"
    p.write_text("# schema: scan_csv_v1\nT_MeV,muq_MeV,muB_MeV,xi\n120.0,0.0,0.0,0.0\n130.0,0.0,0.0,0.2\nbad\n")
    assert read_existing_keys(str(p)) == {(120.0, 0.0, 0.0), (130.0, 0.0, 0.2)}
    assert read_existing_keys(str(tmp_path / "none.csv")) == set()


def test_scan_resume_skips_existing_rows(tmp_path):
    """A second run of the scan appends only the missing keys (run_gap_transport_scan.jl:365-422)."""
    from julia_relaxtime_gb300.scan import run_gap_transport_scan
    from oracle_adapter import oracle_point_solver

    out = tmp_path / "gap.csv"
    opts = ScanOptions(output=str(out), xi_values=[0.0], tmin_mev=120, tmax_mev=140, tstep_mev=10,
                       mubmin_mev=0, mubmax_mev=0, mubstep_mev=60)
    run_gap_transport_scan(opts, solver=oracle_point_solver(12, 6))
    lines = [ln for ln in out.read_text().splitlines() if not ln.startswith("#")]
    assert len(lines) == 4
    opts.tmax_mev = 150
    run_gap_transport_scan(opts, solver=oracle_point_solver(12, 6))
    lines = [ln for ln in out.read_text().splitlines() if not ln.startswith("#")]
    assert len(lines) == 5 and lines[-1].startswith("150.0,")
