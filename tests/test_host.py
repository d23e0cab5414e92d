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


def test_julia_string_fast_path_matches_general():
    """julia_string returns repr for 1e-4 <= |x| < 1e6; the general digit-by-digit routine
    gives the same text there, on random doubles of every magnitude and at the edges."""
    from julia_relaxtime_gb300.scan import _julia_string_general

    rng = np.random.default_rng(3)
    xs = np.concatenate([
        rng.uniform(-1, 1, 20000) * 10.0 ** rng.integers(-8, 9, 20000),
        rng.standard_normal(5000),
        np.array([1e-4, -1e-4, np.nextafter(1e-4, 0), np.nextafter(1e-4, 1), 1e6, np.nextafter(1e6, 0),
                  999999.9999999999, 0.1, 0.2, 0.3, 1.0 / 3.0, 123456.7, 5e-324, 1.7976931348623157e308]),
    ])
    for x in xs:
        assert julia_string(float(x)) == _julia_string_general(float(x)), x


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


def test_scan_rho_norm_uses_profile_rho0_and_batches_xi():
    """rho_norm = rho_baryon / rho0 of the loaded profile (run_gap_transport_scan.jl:497-500), and
    every xi's columns of one temperature go to the solver together (at most two calls per T)."""
    import dataclasses

    from julia_relaxtime_gb300.constants import PNJLParams
    from julia_relaxtime_gb300.scan import scan_rows
    from oracle_adapter import oracle_point_solver

    base = oracle_point_solver(12, 6)
    calls = []

    def solver(T, mu, xi, seeds, max_iter):
        calls.append((float(T[0]), len(T), seeds is None))
        return base(T, mu, xi, seeds, max_iter)

    params = dataclasses.replace(PNJLParams.default(), rho0=0.17)
    opts = ScanOptions(xi_values=[0.0, 0.2], tmin_mev=120, tmax_mev=140, tstep_mev=10, mubmin_mev=0,
                       mubmax_mev=600, mubstep_mev=300, params=params)
    rows = scan_rows(opts, solver)
    assert len(rows) == 2 * 3 * 3
    # reference order: xi -> muB -> T
    keys = [(r["xi"], r["muB_MeV"], r["T_MeV"]) for r in rows]
    assert keys == sorted(keys)
    # T = 120: one MultiSeed call for all 6 columns; later T: one continuation call each
    assert calls[0][1:] == (6, True) and all(c[1:] == (6, False) for c in calls[1:]) and len(calls) == 3
    for r in rows:
        assert r["rho_norm"] == r["rho_baryon"] / 0.17
    default_rows = scan_rows(dataclasses.replace(opts, params=None), base)
    for a, b in zip(rows, default_rows):
        assert b["rho_norm"] == b["rho_baryon"] / 0.16 and a["rho_baryon"] == b["rho_baryon"]


# ---- TmuScan driver (TmuScan.jl) with the oracle as the point solver --------------------
def _tmu_rows(Ts, solver):
    from julia_relaxtime_gb300 import scan

    return scan.tmu_scan_rows(Ts, np.arange(0.0, 401.0, 10.0), [0.0], solver,
                              boundary_path=os.path.join(GOLDEN, "boundary.csv"),
                              cep_path=os.path.join(GOLDEN, "cep.csv"))


def test_tmu_scan_oracle_matches_golden_rows():
    """run_tmu_scan's candidate order, continuation and phase-aware switch (TmuScan.jl:120-301)
    reproduce the stored tmu_scan.csv (p24/t8) at its 6 decimals.  The stored file predates the
    phase-aware tracker: where it stays on the metastable branch past mu_c, the scan here
    switches to the stable one (higher pressure) -- allowed, and checked to be the stable one."""
    from julia_relaxtime_gb300 import scan
    from oracle_adapter import oracle_point_solver

    Ts = [50.0, 100.0, 130.0, 150.0, 200.0]
    rows, stats = _tmu_rows(Ts, oracle_point_solver(24, 8))
    assert stats == {"total": 205, "success": 205, "failure": 0, "skipped": 0}
    g = {(float(r["T_MeV"]), float(r["mu_MeV"])): r for r in read_csv("tmu_scan.csv")}
    switched = 0
    for T, mu, xi, r, msg in rows:
        gr = g[(T, mu)]
        d = max(abs(float(scan._fmt6(r["x"][k])) - float(gr[c]))
                for k, c in enumerate(("phi_u", "phi_d", "phi_s", "Phi1", "Phi2")))
        dp = float(scan._fmt6(r["pressure"])) - float(gr["pressure_fm4"])
        if d <= 2e-6 and abs(dp) <= 2e-6:
            continue
        assert dp > 1e-4, (T, mu, d, dp)  # a different branch only if it is the stable one
        switched += 1
    assert switched <= 2


def test_tmu_csv_format_and_resume(tmp_path):
    from julia_relaxtime_gb300 import scan
    from oracle_adapter import oracle_point_solver

    out = tmp_path / "tmu.csv"
    solver = oracle_point_solver(12, 4)
    st = scan.run_tmu_scan(T_values=[60.0, 180.0], mu_values=[0.0, 10.0, 20.0], output_path=str(out),
                           p_num=12, t_num=4, solver=solver, use_phase_aware=False)
    assert st["total"] == 6 and st["success"] == 6
    lines = out.read_text().splitlines()
    assert lines[0].split(",") == scan.TMU_HEADER and len(scan.TMU_HEADER) == 19
    first = lines[1].split(",")
    assert first[:3] == ["60.000000", "0.000000", "0.000000"] and first[17] == "true"
    assert all(len(c.split(".")[1]) == 6 for c in first[3:15])
    # resume: a second call with one more mu solves only the new points
    st2 = scan.run_tmu_scan(T_values=[60.0, 180.0], mu_values=[0.0, 10.0, 20.0, 30.0], output_path=str(out),
                            p_num=12, t_num=4, solver=solver, use_phase_aware=False)
    assert st2["skipped"] == 6 and st2["success"] == 2
    assert len(out.read_text().splitlines()) == 1 + 8
    # a failed point (the reference's `nothing` result) is written with NaNs and the messages
    row = scan.format_tmu_row(50.0, 10.0, 0.0, None, "seed[hadron] failed")
    c = row.split(",")
    assert c[3] == "NaN" and c[15] == "-1" and c[17] == "false" and c[18] == '"seed[hadron] failed"'
    assert scan._fmt6(float("nan")) == "NaN" and scan._fmt6(-1e-9) == "-0.000000"


# ---- learned-seed verification map (host logic) -----------------------------------------
def test_coexistence_map_flags_coexistence_and_jumps():
    from julia_relaxtime_gb300.learned_seed import TrainConfig, coexistence_map

    cfg = TrainConfig(T_MeV=(50.0, 300.0, 6), mu_MeV=(0.0, 400.0, 6), xi=(-0.5, 0.5, 3))
    nT, nm, nx = 6, 6, 3
    N = nT * nm * nx
    base = np.tile(np.array([-1.8, -1.8, -2.2, 0.01, 0.01]), (N, 1))
    R = np.repeat(base[:, None, :], 6, axis=1).copy()
    Om = np.full((N, 6), -21.0)
    idx = lambda i, j, k: (i * nm + j) * nx + k  # noqa: E731
    # node (1, 4, 0): a second phase 0.01 above the minimum -> flagged
    R[idx(1, 4, 0), 2] = [-0.2, -0.2, -2.0, 0.05, 0.06]
    Om[idx(1, 4, 0), 2] = -20.99
    # node (4, 1, 2): a far-off root 3.5 above the minimum -> not a competing phase
    R[idx(4, 1, 2), 3] = [-5.3, -5.3, -2.3, 0.0, 0.0]
    Om[idx(4, 1, 2), 3] = -17.5
    lab = {"x": base.copy(), "converged": np.ones(N, bool)}
    vm = coexistence_map(None, cfg, lab, roots=(R, Om), grow=0)
    assert vm.flags.shape == (5, 5, 2)
    assert vm.flags[0:2, 3:5, 0].all() and vm.flags.sum() == 4  # the 4 cells around node (1, 4, 0)
    # a jump of the labelled solution along mu between nodes (3, 2, *) and (3, 3, *)
    lab2 = {"x": base.copy(), "converged": np.ones(N, bool)}
    for k in range(nx):
        lab2["x"][idx(3, 3, k), 0] = -0.2
    R2 = np.repeat(lab2["x"][:, None, :], 6, axis=1)
    vm2 = coexistence_map(None, cfg, lab2, roots=(R2, np.full((N, 6), -21.0)), grow=0)
    assert vm2.flags[2:4, 1:4, :].all()
    vm3 = coexistence_map(None, cfg, lab2, roots=(R2, np.full((N, 6), -21.0)), grow=1)
    assert vm3.flags.sum() > vm2.flags.sum()
    assert vm.lo[0] == pytest.approx(50.0 / HBARC) and vm.hi[2] == 0.5


# ---- sharding of the bench over ranks (gloo, world size 2) ---------------------------------
def _shard_worker(rank, world, port, n, q):
    import torch
    import torch.distributed as dist

    from julia_relaxtime_gb300.engine import shard_points

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    mine = shard_points(n, rank, world)
    counts = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(counts, torch.tensor([mine.size], dtype=torch.int64))
    total = torch.tensor([int(mine.sum())], dtype=torch.int64)
    dist.all_reduce(total)
    t = torch.tensor([float(10 + rank)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    q.put((rank, [int(c.item()) for c in counts], int(total.item()), float(t.item())))
    dist.destroy_process_group()


def test_shard_points_two_ranks_gloo():
    """The bench's sharding: every point on exactly one rank, max-over-ranks timing (gloo)."""
    import multiprocessing as mp
    import socket

    from julia_relaxtime_gb300.engine import shard_points

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    n = 589_824 + 3
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_shard_worker, args=(r, 2, port, n, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, counts, total, tmax in res:
        assert sum(counts) == n and abs(counts[0] - counts[1]) <= 1
        assert total == n * (n - 1) // 2  # disjoint and complete
        assert tmax == 11.0
    a, b = shard_points(10, 0, 2), shard_points(10, 1, 2)
    assert set(a) | set(b) == set(range(10)) and not set(a) & set(b)
    with pytest.raises(ValueError):
        shard_points(10, 2, 2)


def test_bench_slices_and_workload_grids():
    """The bench's slices partition each rank's shard; the lazily decoded first-order grid
    (2048 x 2048 x 9, mu_s = mu_u / 2) is the meshgrid of its axes, T slowest and xi fastest;
    the 2^20-point set is reproducible."""
    import bench
    from julia_relaxtime_gb300.engine import shard_points

    n, world, chunks = 1000 + 7, 2, 13
    for rank in range(world):
        mine = shard_points(n, rank, world)
        parts = [bench.slice_indices(n, rank, world, chunks, c) for c in range(chunks)]
        assert np.array_equal(np.sort(np.concatenate(parts)), mine)
        assert np.array_equal(parts[3], mine[3::chunks])
    g = bench.workload_grid("first_order_2048x2048x9")
    assert g["n"] == 2048 * 2048 * 9 and bench.seed_count(g) == 8
    idx = np.array([0, 1, 8, 9, 2048 * 9 - 1, 2048 * 9, 123_456_7, g["n"] - 1])
    T, mu_u, mu_s, xi = g["at"](idx)
    iT, im, ix = np.unravel_index(idx, (2048, 2048, 9))
    np.testing.assert_allclose(T * HBARC, np.linspace(20.0, 150.0, 2048)[iT], rtol=1e-14)
    np.testing.assert_allclose(mu_u * HBARC, np.linspace(250.0, 450.0, 2048)[im], rtol=1e-14)
    np.testing.assert_array_equal(mu_s, 0.5 * mu_u)
    np.testing.assert_allclose(xi, np.round(np.arange(-0.4, 0.4001, 0.1), 10)[ix])
    a, b = bench.workload_grid("surrogate_eval_2p20"), bench.workload_grid("surrogate_eval_2p20")
    assert a["n"] == 1 << 20
    pa, pb = a["at"](np.arange(0, a["n"], 4099)), b["at"](np.arange(0, b["n"], 4099))
    for u, v in zip(pa, pb):
        np.testing.assert_array_equal(u, v)
    assert 50.0 <= pa[0].min() * HBARC and pa[0].max() * HBARC <= 300.0 and np.abs(pa[3]).max() <= 0.5


def test_training_box_of_the_first_order_scan():
    """The label grid of a flavour-asymmetric box (mu_s = mu_u / 2) solves at (mu, mu, mu/2),
    its table holds the MultiSeed candidates plus the extra rows, and the network's inputs are
    scaled to [-1, 1] over the box (the default box: the constants of the 50-300 / 0-400 MeV,
    xi +-0.5 grid)."""
    from julia_relaxtime_gb300 import pnjl
    from julia_relaxtime_gb300.learned_seed import TrainConfig, box_scaling, flavour_mu, grid_points, label_table

    cfg = TrainConfig(T_MeV=(20.0, 150.0, 4), mu_MeV=(250.0, 450.0, 3), xi=(-0.5, 0.5, 2), mu_s_ratio=0.5,
                      label_extra=(pnjl.MEDIUM_SEED_5, pnjl.HIGH_DENSITY_SEED_5))
    T, mu, xi = grid_points(cfg)
    assert T.size == 24 and mu.ndim == 1
    m3 = flavour_mu(cfg, mu)
    np.testing.assert_array_equal(m3[:, 0], mu)
    np.testing.assert_array_equal(m3[:, 1], mu)
    np.testing.assert_array_equal(m3[:, 2], 0.5 * mu)
    assert flavour_mu(TrainConfig(), mu).ndim == 1  # mu_u = mu_d = mu_s: one array
    cold, hot = label_table(cfg)
    assert cold.shape == (8, 5) and hot.shape == (8, 5)
    np.testing.assert_array_equal(cold[6], pnjl.MEDIUM_SEED_5)
    np.testing.assert_array_equal(cold[:6], pnjl.multiseed_table(6)[0])
    shift, scale = box_scaling(cfg)
    lo = np.array([20.0 / HBARC, 250.0 / HBARC, -0.5])
    hi = np.array([150.0 / HBARC, 450.0 / HBARC, 0.5])
    np.testing.assert_allclose((lo - shift) / scale, -1.0, rtol=1e-14)
    np.testing.assert_allclose((hi - shift) / scale, 1.0, rtol=1e-14)
    s0, c0 = box_scaling(TrainConfig())
    np.testing.assert_allclose(s0, [175.0 / HBARC, 200.0 / HBARC, 0.0], rtol=1e-14, atol=1e-15)
    np.testing.assert_allclose(c0, [125.0 / HBARC, 200.0 / HBARC, 0.5], rtol=1e-14)


def test_candidates_and_labels_select_like_solve_multi():
    """The one-launch labels: every candidate alone as a per-point seed, then per point the
    converged candidate of lowest Omega, the earliest among Omegas within the tie tolerance
    (solve_multi, ImplicitSolver.jl:532-559); hot rows at T >= 300 MeV."""
    from julia_relaxtime_gb300.learned_seed import TrainConfig, candidates_and_labels

    cfg = TrainConfig(T_MeV=(250.0, 300.0, 2), mu_MeV=(0.0, 100.0, 2), xi=(0.0, 0.0, 1), label_seeds=3)
    N, S = 4, 3
    om = np.array([[-5.0, -5.0, -7.0, np.nan], [-6.0, -5.0 - 1e-13, -7.5, -1.0], [-6.0, -4.0, -7.5 + 1e-14, -2.0]])
    conv = ~np.isnan(om)

    class FakeEngine:
        def solve(self, T, mu, xi, *, seed_table, seed_table_hot, point_seeds, opts):
            assert T.size == S * N and point_seeds.shape == (S * N, 5) and not opts.auto_multiseed_fallback
            self.seeds = point_seeds.reshape(S, N, 5)
            x = np.repeat(np.arange(S * N, dtype=float)[:, None], 5, axis=1)
            return {"converged": conv.ravel(), "x": x, "omega": np.nan_to_num(om, nan=0.0).ravel()}

    eng = FakeEngine()
    R, Om, lab = candidates_and_labels(eng, cfg)
    assert R.shape == (N, S, 5) and Om.shape == (N, S)
    # point 0: seed 1 (-6) beats seed 0 (-5), seed 2 ties seed 1 -> seed 1; point 1: seed 1 is
    # within the tie of seed 0 -> seed 0; point 2: seed 1; point 3: seed 2 (-2 < -1)
    assert list(lab["x"][:, 0].astype(int)) == [1 * N + 0, 0 * N + 1, 1 * N + 2, 2 * N + 3]
    assert lab["converged"].all()
    # the hot table's rows at T = 300 MeV (points 2, 3 of the T-major grid)
    from julia_relaxtime_gb300.learned_seed import label_table

    table, hot = label_table(cfg)
    assert np.array_equal(eng.seeds[:, 0], table) and np.array_equal(eng.seeds[:, 3], hot)


def test_bench_reference_arm_json_line():
    """bench.py --impl reference (the reference algorithm on the host cores, no GPU) prints one
    JSON line with the bench contract's keys: the metric, whole-job value, timing fields (warm-up
    raised to 3), the CPU baseline it measured and an e2e block without host-device copies."""
    import json
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1",
                          "--cpu-sample", "4"], cwd=root, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = [s for s in out.stdout.splitlines() if s.startswith("{")][-1]
    d = json.loads(line)
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "solves/s" and d["higher_is_better"]
    assert d["steps"] == 1 and d["warmup"] >= 3 and d["vs_baseline"] is None
    assert d["config"]["workload"] == "first_order_2048x2048x9"
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert cb["single_thread"]["cores"] == 1 and cb["single_thread"]["value"] > 0
    assert d["e2e"] == {"value": d["value"], "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
