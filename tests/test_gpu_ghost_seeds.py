"""Verification seeds on spinodal ghosts and near-singular metastable roots.

Points of the first-order box (mu_s = mu_u / 2, p128 x t32, the 8 first-order seed candidates)
where some MultiSeed candidates run into a spinodal ghost: a state just past the point where a
metastable root merges with the unstable branch, where |grad Omega| has a minimum of ~1e-6 and
there is no root.  The oracle's FP64 Newton from those seeds stalls at that residual for all
40 iterations and its trust-region fallback fails too (checked on the oracle when the points
were chosen; the candidates' plateau residuals were 5e-7 .. 1e-5).  At (111.514, 339.301, 0.3)
the candidates instead reach a real, nearly singular metastable root 1.1e-3 fm^-4 above the
minimum.  Each was, alone, the slowest point of a bench step.

Verification mode (every candidate judges the per-point seed) must select exactly what the
plain FP64 MultiSeed solve selects, whether the per-point seed reaches the minimum (the
candidates then carry its Omega as a bound and are dropped on the plateau or by the
float-float Omega prune) or starts on the ghost itself (the per-point seed gives up on the
plateau and the MultiSeed candidates decide).
"""
import numpy as np
import pytest

from julia_relaxtime_gb300 import pnjl
from julia_relaxtime_gb300.engine import SolveOptions
from julia_relaxtime_gb300.pnjl import multiseed_table

pytestmark = pytest.mark.gpu
HBARC = 197.327

# (T, mu_u) in MeV, xi; and the state where the oracle's stalled candidates ended (rounded)
POINTS = [
    ((83.190, 361.480, 0.3), (-1.457457, -1.457457, -2.174958, 0.058687, 0.095563)),
    ((66.551, 316.830, -0.3), (-0.497633, -0.497633, -2.084899, 0.072391, 0.097636)),
    ((51.436, 361.578, 0.3), (-0.71429, -0.71429, -2.09908, 0.045882, 0.060079)),
    ((141.617, 250.195, -0.3), (-0.993413, -0.993413, -2.072509, 0.310026, 0.338789)),
    ((135.965, 272.667, -0.2), (-1.113789, -1.113789, -2.10164, 0.260387, 0.295186)),
    ((54.231, 361.187, 0.3), (-0.716125, -0.716125, -2.099197, 0.048998, 0.06461)),
    ((91.827, 339.204, 0.1), (-0.6767, -0.6767, -2.093468, 0.114943, 0.149852)),
    ((111.514, 339.301, 0.3), (-1.244294, -1.244294, -2.143496, 0.132164, 0.176222)),
]


def _points():
    T = np.array([p[0][0] for p in POINTS]) / HBARC
    mu = np.array([p[0][1] for p in POINTS]) / HBARC
    xi = np.array([p[0][2] for p in POINTS])
    ghost = np.array([p[1] for p in POINTS])
    return T, np.stack([mu, mu, 0.5 * mu], axis=1), xi, ghost


def _same_selection(r, ref):
    assert r["converged"].all() and ref["converged"].all()
    np.testing.assert_allclose(r["omega"], ref["omega"], rtol=1e-12, atol=0)
    phi = np.abs(r["x"][:, :3] - ref["x"][:, :3]).max(axis=1) / np.abs(ref["x"][:, :3]).max(axis=1)
    assert phi.max() <= 1e-9
    assert np.abs(r["x"][:, 3:] - ref["x"][:, 3:]).max() <= 1e-10


@pytest.mark.parametrize("start", ["minimum", "ghost"])
def test_verification_on_ghost_points_matches_multiseed(engine_factory, start):
    eng = engine_factory(128, 32)
    T, mu, xi, ghost = _points()
    table, hot = multiseed_table(6, (pnjl.MEDIUM_SEED_5, pnjl.HIGH_DENSITY_SEED_5))
    ref = eng.solve(T, mu, xi, seed_table=table, seed_table_hot=hot,
                    opts=SolveOptions(iterations=40, ftol=1e-10, precision="fp64"))
    if start == "minimum":
        seeds = ref["x"] * (1.0 + 1e-3)  # in the minimum's basin: the candidates get its Omega as bound
    else:
        seeds = ghost.copy()  # on the ghost: the per-point seed stalls and gives up
    opts = SolveOptions(iterations=40, ftol=1e-10, precision="mixed", verify_seeds=table.shape[0],
                        verify_T_max_MeV=1000.0)
    r = eng.solve(T, mu, xi, seed_table=table, seed_table_hot=hot, point_seeds=seeds, opts=opts)
    st = eng.stats()
    _same_selection(r, ref)
    print(f"{start}: pruned {st['pruned_candidates']}, rescues {st['fp64_rescues']}, "
          f"chosen {r['chosen_seed'].tolist()}, last kernel {st['last_kernel_ms']:.1f} ms")
    # the candidates stalled on a ghost, or on the metastable root above the bound, are dropped
    assert st["pruned_candidates"] > 0
    if start == "minimum":
        assert (r["chosen_seed"] == -1).all()  # the per-point root is the minimum and is kept


def test_ghost_points_identical_across_launch_forms(engine_factory):
    """The rules for slow seeds -- the learned seed's give-up, the plateau test with the per-point
    root or seed 0's Omega as bound -- depend only on values fixed per point, never on which
    seed finishes first: the same results, bit for bit, from every launch form (the fused
    kernel with 0 or 2 certifying warps, the two kernels, the chunk pipeline) and over repeats.
    Each point is solved from its ghost (fallback mode: the MultiSeed candidates with seed 0's
    bound) and from its minimum (verification mode: the per-point root as bound)."""
    eng = engine_factory(128, 32)
    T, mu, xi, ghost = _points()
    table, hot = multiseed_table(6, (pnjl.MEDIUM_SEED_5, pnjl.HIGH_DENSITY_SEED_5))
    ref = eng.solve(T, mu, xi, seed_table=table, seed_table_hot=hot,
                    opts=SolveOptions(iterations=40, ftol=1e-10, precision="fp64"))
    # every point twice, once per start, in one batch
    T2, mu2, xi2 = np.concatenate([T, T]), np.concatenate([mu, mu]), np.concatenate([xi, xi])
    seeds = np.concatenate([ghost, ref["x"] * (1.0 + 1e-3)])
    opts = SolveOptions(iterations=40, ftol=1e-10, precision="mixed", verify_seeds=table.shape[0],
                        verify_T_max_MeV=1000.0)
    outs = []
    for chunks, cert in ((1, 0), (1, 2), (-1, 0), (2, 0), (1, 0)):
        eng.set_tuning(32, 0, pipeline_chunks=chunks, cert_warps=cert)
        outs.append(eng.solve(T2, mu2, xi2, seed_table=table, seed_table_hot=hot, point_seeds=seeds, opts=opts))
        assert eng.stats()["device_wait_timeouts"] == 0
    eng.set_tuning(32, 0, pipeline_chunks=0, cert_warps=0)
    for r in outs[1:]:
        for k in ("x", "omega", "entropy", "n_q", "status", "chosen_seed", "iterations", "converged"):
            np.testing.assert_array_equal(r[k], outs[0][k], err_msg=k)
    n = T.size
    for half in (slice(0, n), slice(n, 2 * n)):
        r = {k: v[half] for k, v in outs[0].items()}
        _same_selection(r, ref)
