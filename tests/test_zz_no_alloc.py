"""pnjl_solve_batch_noalloc: the allocation-free solve, checked against pnjl_solve_batch_device.

Some callers of this library cannot allocate device memory when they solve -- hosts whose
device memory is owned by another allocator's pool that must account for every byte, and
services that reserve all memory at start-up so that no later call can fail for lack of it.  The no-alloc entry point serves them: its
scratch is a static device array of fixed size.  This test drives it through the C ABI with
device buffers owned by the test, several calls in a row (the shared scratch keeps the
previous call's contents, so the later calls show that each call starts clean), and compares every
output with the allocating entry point on the same inputs, at the parity tolerance of the
GPU tests (the two run the same kernel, so agreement is in fact exact).

The file name sorts last so that a run stopping at the first failure has run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HBARC = 197.327
FIELDS_F64 = {"x": 5, "omega": 1, "pressure": 1, "rho_norm": 1, "entropy": 1, "energy": 1, "residual_norm": 1,
              "masses": 3, "rho": 3, "n_q": 3, "n_aq": 3}
FIELDS_I32 = ("iterations", "chosen_seed", "status")


def _device_outputs(torch, n, dev):
    out = {k: torch.full((n * w,), float("nan"), dtype=torch.float64, device=dev) for k, w in FIELDS_F64.items()}
    for k in FIELDS_I32:
        out[k] = torch.full((n,), -7, dtype=torch.int32, device=dev)
    out["converged"] = torch.full((n,), 9, dtype=torch.uint8, device=dev)
    return out


def _soa(api, out):
    soa = api.pnjl_result_soa()
    for k, v in out.items():
        ptr_t = api.i32p if k in FIELDS_I32 else (api.u8p if k == "converged" else api.dp)
        setattr(soa, k, C.cast(C.c_void_p(v.data_ptr()), ptr_t))
    return soa


def _compare(ref, got, n):
    for k in FIELDS_F64:
        a = ref[k].cpu().numpy()
        b = got[k].cpu().numpy()
        np.testing.assert_allclose(b, a, rtol=1e-12, atol=1e-14, err_msg=k)
    for k in FIELDS_I32 + ("converged",):
        assert np.array_equal(ref[k].cpu().numpy(), got[k].cpu().numpy()), k


def _noalloc_call(api, lib, params, p_num, t_num, n, T, mu, mus, xi, o, got, stream):
    soa = _soa(api, got)
    cast = lambda t: C.cast(C.c_void_p(t.data_ptr()), api.dp)  # noqa: E731
    return lib.pnjl_solve_batch_noalloc(C.byref(params), p_num, t_num, 10.0, n, cast(T), cast(mu), cast(mu),
                                        cast(mus), cast(xi), C.byref(o), C.byref(soa),
                                        C.c_void_p(stream.cuda_stream))


def test_noalloc_matches_allocating_entry_point_twice():
    """Two calls in a row, the second at another quadrature order (the node tables in the
    shared array are reloaded), then a call with one device seed per point
    (PNJL_SEEDS_PER_POINT: no per-point completion counters are cleared in that mode)."""
    torch = pytest.importorskip("torch")
    from julia_relaxtime_gb300 import _capi as api
    from julia_relaxtime_gb300.engine import GapEngine, SolveOptions
    from julia_relaxtime_gb300.pnjl import multiseed_table

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    eng = GapEngine(device=0, p_num=32, t_num=8)
    lib = api.lib()
    params = eng.params.to_c()
    table, hot = multiseed_table(4)
    opts = SolveOptions(iterations=40, ftol=1e-10)
    rng = np.random.default_rng(17)
    stream = torch.cuda.current_stream(dev)
    for call, (n, p_num, t_num, per_point) in enumerate(((96, 32, 8, False), (61, 24, 6, False),
                                                         (77, 24, 6, True))):
        eng.set_nodes(p_num, t_num)
        T = torch.tensor(rng.uniform(40, 320, n) / HBARC, dtype=torch.float64, device=dev)
        mu = torch.tensor(rng.uniform(0, 420, n) / HBARC, dtype=torch.float64, device=dev)
        mus = (0.5 * mu).contiguous()
        xi = torch.tensor(rng.uniform(-0.5, 0.5, n), dtype=torch.float64, device=dev)
        seeds = None
        if per_point:
            # one MultiSeed row per point, chosen at random; the table stays the fallback
            rows = rng.integers(0, table.shape[0], n)
            seeds = torch.tensor(table[rows].reshape(-1), dtype=torch.float64, device=dev)
        # the allocating entry point (pnjl_solve_batch_device) as the reference answer
        ref = _device_outputs(torch, n, dev)
        torch.cuda.synchronize()
        eng.solve_device(n, T.data_ptr(), mu.data_ptr(), mu.data_ptr(), mus.data_ptr(), xi.data_ptr(),
                         {k: v.data_ptr() for k, v in ref.items()}, seed_table=table, seed_table_hot=hot, opts=opts,
                         d_point_seeds=seeds.data_ptr() if per_point else 0)
        eng.synchronize()
        # the allocation-free entry point on the test's stream
        got = _device_outputs(torch, n, dev)
        o = eng._opts_struct(opts, table, hot, 300.0, per_point, seeds.data_ptr() if per_point else None)
        rc = _noalloc_call(api, lib, params, p_num, t_num, n, T, mu, mus, xi, o, got, stream)
        assert rc == api.PNJL_OK, (call, rc)
        stream.synchronize()
        _compare(ref, got, n)
        assert got["status"].cpu().numpy().max() <= api.PNJL_POINT_ALL_SEEDS_FAILED
        assert got["converged"].cpu().numpy().sum() >= n - 2, call
    eng.close()


def test_noalloc_rejects_mixed_precision():
    """The fixed scratch holds the FP64 solver's records only: a mixed-precision request is an
    error, not a silent FP64 solve; the output buffers stay untouched."""
    torch = pytest.importorskip("torch")
    from julia_relaxtime_gb300 import _capi as api
    from julia_relaxtime_gb300.constants import PNJLParams
    from julia_relaxtime_gb300.engine import GapEngine, SolveOptions
    from julia_relaxtime_gb300.pnjl import multiseed_table

    dev = torch.device("cuda", 0)
    lib = api.lib()
    params = PNJLParams.default().to_c()
    table, hot = multiseed_table(4)
    n = 8
    T = torch.full((n,), 100.0 / HBARC, dtype=torch.float64, device=dev)
    mu = torch.full((n,), 200.0 / HBARC, dtype=torch.float64, device=dev)
    xi = torch.zeros(n, dtype=torch.float64, device=dev)
    got = _device_outputs(torch, n, dev)
    o = GapEngine._opts_struct(SolveOptions(precision="mixed"), table, hot, 300.0, False, None)
    rc = _noalloc_call(api, lib, params, 32, 8, n, T, mu, mu, xi, o, got, torch.cuda.current_stream(dev))
    assert rc == api.PNJL_ERR_INVALID_ARGUMENT
    torch.cuda.synchronize()
    assert np.all(got["status"].cpu().numpy() == -7)


def test_noalloc_rejects_batches_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    from julia_relaxtime_gb300 import _capi as api
    from julia_relaxtime_gb300.constants import PNJLParams
    from julia_relaxtime_gb300.engine import GapEngine, SolveOptions
    from julia_relaxtime_gb300.pnjl import multiseed_table

    lib = api.lib()
    params = PNJLParams.default().to_c()
    table, hot = multiseed_table(4)
    o = GapEngine._opts_struct(SolveOptions(), table, hot, 300.0, False, None)
    n = api.PNJL_NOALLOC_MAX_TASKS // 4 + 1  # 4 seeds per point -> one task too many
    dummy = C.cast(C.c_void_p(16), api.dp)    # never dereferenced: the size check comes first
    soa = api.pnjl_result_soa()
    rc = lib.pnjl_solve_batch_noalloc(C.byref(params), 32, 8, 10.0, n, dummy, dummy, dummy, dummy, dummy,
                                      C.byref(o), C.byref(soa), None)
    assert rc == api.PNJL_ERR_TOO_LARGE
    rc = lib.pnjl_solve_batch_noalloc(C.byref(params), 32, 8, 10.0, 0, None, None, None, None, None,
                                      C.byref(o), C.byref(soa), None)
    assert rc == api.PNJL_OK
