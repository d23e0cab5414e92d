"""The fused kernel's bounded waits (pnjl_set_wait_limits), exercised without a GPU fault.

In the fused mixed-precision kernel a warp that takes a listed point's verification task
polls that slot's ready flag, written by the running warp that listed the point, and a seed
whose FP32 root an earlier seed is still certifying polls that verdict.  Both waits are
bounded.  With the bounds set to 0 polls a ready flag not set at the first read gives up at
once: the task is left undone, counted in device_wait_timeouts, and the host-array solve
returns an error instead of incomplete results.  The test checks that the kernel always
finishes, that the error is raised exactly when a wait ran out (and the results are right
otherwise), and that the same context solves correctly again with the default bounds.
"""
import time

import numpy as np
import pytest

from julia_relaxtime_gb300 import _capi as api
from julia_relaxtime_gb300.learned_seed import LearnedSeed, default_learned_opts
from julia_relaxtime_gb300.pnjl import MultiSeed, multiseed_table
from julia_relaxtime_gb300.engine import SolveOptions

pytestmark = pytest.mark.gpu
HBARC = 197.327


def test_wait_limits_bound_the_fused_kernel_waits(engine_factory):
    eng = engine_factory(32, 8)
    assert eng.wait_limits() == (1 << 24, 1 << 20)
    rng = np.random.default_rng(41)
    n = 6000
    T = rng.uniform(40, 160, n) / HBARC
    mu = rng.uniform(200, 420, n) / HBARC
    xi = rng.uniform(-0.4, 0.4, n)
    # a network trained briefly on MultiSeed roots of a few points; every point is verified by
    # all candidates (T below 1000 MeV), so every point is listed and its tasks are taken by
    # other warps while it is being written
    table, hot = multiseed_table(6)
    lab = eng.solve(T[:512], mu[:512], xi[:512], seed_table=table, seed_table_hot=hot,
                    opts=SolveOptions(iterations=40, ftol=1e-10, precision="mixed"))
    ls = LearnedSeed(eng, seed=5)
    ls.default_scaling(lab["x"])
    ls.fit(T[:512], mu[:512], xi[:512], lab["x"], epochs=20, batch=128)
    eng.set_tuning(32, 0, pipeline_chunks=1)  # the fused kernel
    opts = default_learned_opts(ftol=1e-10, verify_T_max_MeV=1000.0)

    def run():
        t0 = time.perf_counter()
        try:
            r = ls.solve(T, mu, xi, opts=opts, multiseed=MultiSeed())
            err = None
        except api.CudaLibraryError as e:
            r, err = None, str(e)
        return r, err, eng.stats()["device_wait_timeouts"], time.perf_counter() - t0

    ref, err, to, t_ref = run()
    assert err is None and to == 0
    eng.set_wait_limits(0, 0)
    assert eng.wait_limits() == (0, 0)
    seen = 0
    for _ in range(4):
        r, err, to, dt = run()
        assert dt < 3.0 * t_ref + 2.0  # no wait outlives its bound
        if to > 0:
            seen += to
            assert err is not None and "gave up waiting" in err
        else:
            assert err is None
            same = np.abs(r["omega"] - ref["omega"]) <= 1e-12 * np.abs(ref["omega"])
            assert same.all() and np.array_equal(r["converged"], ref["converged"])
    print(f"ready waits that ran out with a bound of 0 polls: {seen}")
    eng.set_wait_limits(1 << 24, 1 << 20)
    again, err, to, _ = run()
    assert err is None and to == 0
    np.testing.assert_array_equal(again["x"], ref["x"])
    np.testing.assert_array_equal(again["chosen_seed"], ref["chosen_seed"])
