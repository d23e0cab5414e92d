"""build_K_data on the GPU (pnjl_kdata_batch / pnjl_kdata_batch_device) against the oracle.

The K data are the relaxation-time chain's per-point input (run_gap_transport_scan.jl:297-305):
the one-loop integral A(m_f, mu, T, Phi, Phibar) on 64 Gauss-Legendre nodes of [0, 10]
(OneLoopIntegrals.jl:531-543), G^f (EffectiveCouplings.jl:56-60) and the effective couplings
with their determinants (:112-115, 242-279).  Tolerance: 1e-13 of each field's scale (FP64
on both sides, the same node order; only exp / log / sqrt differ in their last bit).
"""
import numpy as np
import pytest

from julia_relaxtime_gb300 import _capi as api
from julia_relaxtime_gb300.engine import SolveOptions
from julia_relaxtime_gb300.pnjl import multiseed_table
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
HBARC = 197.327


def _compare(got, ref, rtol=1e-13):
    for k in api.KDATA_FIELDS:
        scale = max(np.abs(ref[k]).max(), 1e-300)
        err = np.abs(got[k] - ref[k]).max()
        assert err <= rtol * scale, (k, err, scale)


def test_kdata_of_solved_points_matches_oracle(engine_factory):
    eng = engine_factory(24, 8)
    rng = np.random.default_rng(31)
    n = 300
    T = rng.uniform(20, 320, n) / HBARC
    mu = rng.uniform(0, 450, n) / HBARC
    xi = rng.uniform(-0.4, 0.4, n)
    table, hot = multiseed_table(4)
    res = eng.solve(T, mu, xi, seed_table=table, seed_table_hot=hot, opts=SolveOptions(iterations=40, ftol=1e-10))
    ok = res["converged"]
    assert ok.mean() > 0.97
    P = orc.default_params()
    for p_num, p_max in ((64, 10.0), (128, 20.0)):
        got = eng.kdata(T[ok], mu[ok], mu[ok], res["masses"][ok], res["x"][ok], p_num=p_num, p_max=p_max)
        ref = orc.kdata(P, T[ok], mu[ok], mu[ok], res["masses"][ok], res["x"][ok], p_num=p_num, p_max=p_max)
        _compare(got, ref)
    # flavour-asymmetric chemical potentials (mu_s = mu_u / 2): A_s takes mu_s
    got = eng.kdata(T[ok], mu[ok], 0.5 * mu[ok], res["masses"][ok], res["x"][ok])
    ref = orc.kdata(P, T[ok], mu[ok], 0.5 * mu[ok], res["masses"][ok], res["x"][ok])
    _compare(got, ref)


def test_kdata_device_entry_point_and_edges(engine_factory):
    torch = pytest.importorskip("torch")
    eng = engine_factory(16, 4)
    rng = np.random.default_rng(8)
    n = 1000
    T = rng.uniform(10, 400, n) / HBARC
    mu_u = rng.uniform(-100, 500, n) / HBARC
    mu_s = rng.uniform(0, 300, n) / HBARC
    masses = np.column_stack([rng.uniform(0.0, 2.0, n)] * 2 + [rng.uniform(0.3, 2.5, n)])
    masses[:5, 0] = masses[:5, 1] = 1e-15  # the massless branch of the constant term
    x = np.column_stack([rng.uniform(-2, 0, (n, 3)), rng.uniform(0, 1, (n, 2))])
    host = eng.kdata(T, mu_u, mu_s, masses, x)
    _compare(host, orc.kdata(orc.default_params(), T, mu_u, mu_s, masses, x))
    dev = torch.device("cuda", 0)
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in
         (("T", T), ("mu_u", mu_u), ("mu_s", mu_s), ("masses", masses.ravel()), ("x", x.ravel()))}
    out = {k: torch.full((n,), np.nan, dtype=torch.float64, device=dev) for k in api.KDATA_FIELDS[:8]}
    torch.cuda.synchronize()
    eng.kdata_device(n, t["T"].data_ptr(), t["mu_u"].data_ptr(), t["mu_s"].data_ptr(), t["masses"].data_ptr(),
                     t["x"].data_ptr(), {k: v.data_ptr() for k, v in out.items()})
    eng.synchronize()
    for k, v in out.items():
        assert np.array_equal(v.cpu().numpy(), host[k]), k  # the same kernel: identical bits
    # empty batch, bad node counts
    assert eng.kdata(T[:0], mu_u[:0], mu_s[:0], masses[:0], x[:0])["A_u"].size == 0
    with pytest.raises(api.CudaLibraryError):
        eng.kdata(T, mu_u, mu_s, masses, x, p_num=0)
    with pytest.raises(api.CudaLibraryError):
        eng.kdata(T, mu_u, mu_s, masses, x, p_max=-1.0)
