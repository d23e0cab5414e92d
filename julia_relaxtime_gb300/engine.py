"""GapEngine: host-side owner of one libpnjl_cuda context (one GPU, one stream).

All compute goes through the C ABI (include/pnjl_cuda.h); numpy arrays are the host
containers.  There is no CPU fallback: without the library every call raises.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _capi as api
from .constants import PNJLParams

PRECISIONS = {"fp64": api.PNJL_PREC_FP64, "mixed": api.PNJL_PREC_MIXED}
EVAL_PRECISIONS = dict(PRECISIONS, ff_residual=api.PNJL_PREC_FF_RESIDUAL, fp64_cert=api.PNJL_PREC_FP64_CERT,
                       fp32_newton=api.PNJL_PREC_FP32_NEWTON)


@dataclass
class SolveOptions:
    """Keyword arguments of solve(::FixedMu, ...) (ImplicitSolver.jl:211-223) that reach the GPU.

    ``iterations`` is NLsolve's iteration cap (NLsolve default 1000; the scan script passes 40).
    ``ftol``/``xtol`` are fixed at 1e-9 in the reference (ImplicitSolver.jl:112,144).
    ``omega_tie_rtol``: seeds whose converged Omega lies within rtol*|Omega| of the kept one are
    treated as the same minimum and the earlier seed is kept (0 gives a strict argmin).
    """
    iterations: int = 1000
    ftol: float = 1e-9
    xtol: float = 1e-9
    residual_norm_max: float = 1e-6
    phi_tol: float = 1e-8
    omega_tie_rtol: float = 1e-12
    trust_region_fallback: bool = True
    auto_multiseed_fallback: bool = True
    precision: str = "fp64"
    # per-point seeds only: also try the first `verify_seeds` table rows (-1: all) below this temperature
    verify_seeds: int = 0
    verify_T_max_MeV: float = 170.0
    verify_max_step: float = 0.0
    # ... or, when given, in the flagged cells of this (T, mu_u, xi) map instead of below verify_T_max_MeV
    verify_map: "VerifyMap | None" = None


@dataclass
class VerifyMap:
    """Cells of a uniform (T, mu_u, xi) grid (T, mu in fm^-1) where per-point solutions are
    verified by the MultiSeed candidates (pnjl_solve_opts::verify_map)."""
    flags: np.ndarray  # uint8 [nT, nmu, nxi]
    lo: tuple          # (T, mu, xi) lower edges
    hi: tuple          # upper edges

    def __post_init__(self):
        self.flags = np.ascontiguousarray(np.asarray(self.flags, dtype=np.uint8))
        if self.flags.ndim != 3:
            raise ValueError("verify map flags must be 3-D (T, mu, xi)")

    def fraction(self) -> float:
        return float(self.flags.mean()) if self.flags.size else 0.0


def shard_points(n: int, rank: int, world: int) -> np.ndarray:
    """Indices of the points rank `rank` of `world` solves: a strided shard (points are
    independent, so ranks exchange no data; every point belongs to exactly one rank and
    every rank's share spans the whole (T, mu, xi) box)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    return np.arange(rank, n, world, dtype=np.int64)


def _dp(a):
    return a.ctypes.data_as(api.dp) if a is not None else None


def _f64(a, n=None, shape=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if shape is not None:
        a = np.ascontiguousarray(np.broadcast_to(a, shape))
    elif n is not None and a.ndim == 0:
        a = np.full(n, float(a))
    return a


class BatchResult(dict):
    """Per-point arrays of one batched solve (keys follow pnjl_result_soa)."""

    def __getattr__(self, k):
        try:
            return self[k]
        except KeyError as e:
            raise AttributeError(k) from e


class GapEngine:
    def __init__(self, params: PNJLParams | None = None, device: int = 0, p_num: int = 64, t_num: int = 8,
                 p_max: float = 10.0):
        self._lib = api.lib()
        self.params = params or PNJLParams.default()
        cp = self.params.to_c()
        ctx = C.c_void_p()
        rc = self._lib.pnjl_init(C.byref(cp), device, C.byref(ctx))
        if rc != api.PNJL_OK or not ctx.value:
            raise api.CudaLibraryError(f"pnjl_init failed with code {rc} (device {device})")
        self._ctx = ctx
        self.device = device
        self.p_num = self.t_num = 0
        self.p_max = p_max
        self.set_nodes(p_num, t_num, p_max)

    # -- lifecycle ---------------------------------------------------------------------
    def close(self):
        if getattr(self, "_ctx", None) is not None and self._ctx.value:
            self._lib.pnjl_destroy(self._ctx)
            self._ctx = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc, what):
        api.check(self._ctx, rc, what)

    # -- nodes -------------------------------------------------------------------------
    def set_nodes(self, p_num: int, t_num: int, p_max: float = 10.0):
        if (p_num, t_num, p_max) == (self.p_num, self.t_num, self.p_max):
            return
        self._check(self._lib.pnjl_set_nodes(self._ctx, int(p_num), int(t_num), float(p_max)), "pnjl_set_nodes")
        self.p_num, self.t_num, self.p_max = int(p_num), int(t_num), float(p_max)

    def nodes(self):
        n = self.p_num * self.t_num
        p, c, w = np.zeros(n), np.zeros(n), np.zeros(n)
        self._check(self._lib.pnjl_get_nodes(self._ctx, _dp(p), _dp(c), _dp(w)), "pnjl_get_nodes")
        return p, c, w

    # -- evaluation ----------------------------------------------------------------------
    def _point_arrays(self, T, mu, xi):
        T = _f64(T).reshape(-1)
        n = T.size
        mu = np.asarray(mu, dtype=np.float64)
        if mu.ndim <= 1 and mu.size in (1, n) and not (mu.ndim == 1 and mu.size == 3 and n != 3):
            mu3 = np.repeat(np.broadcast_to(mu.reshape(-1), (n,))[:, None], 3, axis=1)
        else:
            mu3 = np.broadcast_to(mu.reshape(-1, 3), (n, 3))
        mu_u = np.ascontiguousarray(mu3[:, 0])
        mu_d = np.ascontiguousarray(mu3[:, 1])
        mu_s = np.ascontiguousarray(mu3[:, 2])
        xi = _f64(xi, shape=(n,))
        return n, T, mu_u, mu_d, mu_s, xi

    def evaluate(self, x, T, mu, xi, precision: str = "fp64"):
        """Omega, grad_x Omega [n,5], Hessian_x Omega [n,5,5] at given states.  precision
        "ff_residual": the gradient from the float-float pass alone (Omega, Hessian NaN)."""
        n, T, mu_u, mu_d, mu_s, xi = self._point_arrays(T, mu, xi)
        x = _f64(x, shape=(n, 5))
        om, g, h = np.zeros(n), np.zeros((n, 5)), np.zeros((n, 5, 5))
        rc = self._lib.pnjl_eval_batch(self._ctx, n, _dp(x), _dp(T), _dp(mu_u), _dp(mu_d), _dp(mu_s), _dp(xi),
                                       EVAL_PRECISIONS[precision], _dp(om), _dp(g), _dp(h))
        self._check(rc, "pnjl_eval_batch")
        return om, g, h

    def thermo(self, x, T, mu, xi) -> BatchResult:
        n, T, mu_u, mu_d, mu_s, xi = self._point_arrays(T, mu, xi)
        x = _f64(x, shape=(n, 5))
        out = BatchResult(omega=np.zeros(n), pressure=np.zeros(n), rho_norm=np.zeros(n), entropy=np.zeros(n),
                          energy=np.zeros(n), masses=np.zeros((n, 3)), rho=np.zeros((n, 3)), n_q=np.zeros((n, 3)),
                          n_aq=np.zeros((n, 3)))
        soa = api.pnjl_result_soa()
        for k in ("omega", "pressure", "rho_norm", "entropy", "energy", "masses", "rho", "n_q", "n_aq"):
            setattr(soa, k, _dp(out[k]))
        rc = self._lib.pnjl_thermo_batch(self._ctx, n, _dp(x), _dp(T), _dp(mu_u), _dp(mu_d), _dp(mu_s), _dp(xi),
                                         C.byref(soa))
        self._check(rc, "pnjl_thermo_batch")
        return out

    # -- solve -----------------------------------------------------------------------------
    @staticmethod
    def _opts_struct(opts: SolveOptions, seed_table, seed_table_hot, hot_T_MeV, per_point, point_seeds):
        o = api.pnjl_solve_opts()
        o.seed_mode = api.PNJL_SEEDS_PER_POINT if per_point else api.PNJL_SEEDS_TABLE
        o.n_seeds = 0 if seed_table is None else seed_table.shape[0]
        o.seed_table = _dp(seed_table)
        o.seed_table_hot = _dp(seed_table_hot)
        o.hot_T_MeV = hot_T_MeV
        o.point_seeds = _dp(point_seeds) if isinstance(point_seeds, np.ndarray) else (
            C.cast(C.c_void_p(point_seeds), api.dp) if point_seeds else None)
        o.max_iter = int(opts.iterations)
        o.ftol = opts.ftol
        o.xtol = opts.xtol
        o.residual_norm_max = opts.residual_norm_max
        o.phi_tol = opts.phi_tol
        o.omega_tie_rtol = opts.omega_tie_rtol
        o.trust_region_fallback = int(bool(opts.trust_region_fallback))
        o.auto_multiseed_fallback = int(bool(opts.auto_multiseed_fallback))
        o.precision = PRECISIONS[opts.precision]
        o.verify_seeds = o.n_seeds if opts.verify_seeds < 0 else int(opts.verify_seeds)  # -1: every table row
        o.verify_T_max_MeV = float(opts.verify_T_max_MeV)
        o.verify_max_step = float(opts.verify_max_step)
        vm = opts.verify_map
        if vm is not None:
            o.verify_map = vm.flags.ctypes.data_as(api.u8p)
            for k in range(3):
                o.verify_map_dims[k] = int(vm.flags.shape[k])
                o.verify_map_lo[k] = float(vm.lo[k])
                o.verify_map_hi[k] = float(vm.hi[k])
        return o

    def solve(self, T, mu, xi, *, seed_table=None, seed_table_hot=None, hot_T_MeV: float = 300.0,
              point_seeds=None, opts: SolveOptions | None = None, learned: bool = False) -> BatchResult:
        """Batched solve(::FixedMu) over host arrays (synchronous; includes the copies).

        seed_table [S,5]: MultiSeed candidates (min-Omega selection) and the fallback table.
        point_seeds [n,5]: one seed per point (ContinuitySeed-like); None selects table mode.
        learned: the trained network's seed per point, computed on the device
        (pnjl_solve_batch_learned); seed_table is then the fallback and verification table.
        """
        opts = opts or SolveOptions()
        n, T, mu_u, mu_d, mu_s, xi = self._point_arrays(T, mu, xi)
        st = None if seed_table is None else _f64(seed_table).reshape(-1, 5)
        sth = None if seed_table_hot is None else _f64(seed_table_hot).reshape(-1, 5)
        ps = None if point_seeds is None or learned else _f64(point_seeds, shape=(n, 5))
        o = self._opts_struct(opts, st, sth, hot_T_MeV, ps is not None, ps)
        out = BatchResult(
            x=np.zeros((n, 5)), omega=np.zeros(n), pressure=np.zeros(n), rho_norm=np.zeros(n), entropy=np.zeros(n),
            energy=np.zeros(n), masses=np.zeros((n, 3)), rho=np.zeros((n, 3)), n_q=np.zeros((n, 3)),
            n_aq=np.zeros((n, 3)), residual_norm=np.zeros(n), iterations=np.zeros(n, np.int32),
            chosen_seed=np.zeros(n, np.int32), status=np.zeros(n, np.int32), converged=np.zeros(n, np.uint8))
        soa = api.pnjl_result_soa()
        for k, v in out.items():
            ptr_t = api.i32p if v.dtype == np.int32 else (api.u8p if v.dtype == np.uint8 else api.dp)
            setattr(soa, k, v.ctypes.data_as(ptr_t))
        fn = self._lib.pnjl_solve_batch_learned if learned else self._lib.pnjl_solve_batch
        rc = fn(self._ctx, n, _dp(T), _dp(mu_u), _dp(mu_d), _dp(mu_s), _dp(xi), C.byref(o), C.byref(soa))
        self._check(rc, "pnjl_solve_batch_learned" if learned else "pnjl_solve_batch")
        out["converged"] = out["converged"].astype(bool)
        return out

    def solve_device(self, n: int, d_T: int, d_mu_u: int, d_mu_d: int, d_mu_s: int, d_xi: int, d_out: dict, *,
                     seed_table=None, seed_table_hot=None, hot_T_MeV: float = 300.0, d_point_seeds: int = 0,
                     opts: SolveOptions | None = None, learned: bool = False):
        """Asynchronous solve on device pointers (integers); d_out maps result fields to device pointers.
        learned: seeds from the trained network (pnjl_solve_batch_learned_device)."""
        opts = opts or SolveOptions()
        st = None if seed_table is None else _f64(seed_table).reshape(-1, 5)
        sth = None if seed_table_hot is None else _f64(seed_table_hot).reshape(-1, 5)
        ps = None if learned else (d_point_seeds or None)
        o = self._opts_struct(opts, st, sth, hot_T_MeV, ps is not None, ps)
        soa = api.pnjl_result_soa()
        for k, v in d_out.items():
            ptr_t = dict(iterations=api.i32p, chosen_seed=api.i32p, status=api.i32p, converged=api.u8p).get(k, api.dp)
            setattr(soa, k, C.cast(C.c_void_p(v), ptr_t))
        cast = lambda p: C.cast(C.c_void_p(p), api.dp)  # noqa: E731
        fn = self._lib.pnjl_solve_batch_learned_device if learned else self._lib.pnjl_solve_batch_device
        rc = fn(self._ctx, n, cast(d_T), cast(d_mu_u), cast(d_mu_d), cast(d_mu_s), cast(d_xi), C.byref(o),
                C.byref(soa))
        self._check(rc, "pnjl_solve_batch_learned_device" if learned else "pnjl_solve_batch_device")
        self._keep = (st, sth)  # seed tables are read by the async host->device copy

    # -- K data of the relaxation-time chain ------------------------------------------------
    def kdata(self, T, mu_u, mu_s, masses, x, *, p_num: int = 64, p_max: float = 10.0) -> dict:
        """build_K_data (run_gap_transport_scan.jl:297-305) at n solved points, host arrays:
        one-loop A per flavour on p_num Gauss-Legendre nodes of [0, p_max] (the script's 64 on
        [0, 10]), G^f and the effective couplings.  masses [n,3] and x [n,5] as a solve returns
        them.  Returns {field: [n]} over _capi.KDATA_FIELDS."""
        T = _f64(np.atleast_1d(T))
        n = T.size
        mu_u = _f64(np.broadcast_to(np.asarray(mu_u, dtype=np.float64), (n,)))
        mu_s = _f64(np.broadcast_to(np.asarray(mu_s, dtype=np.float64), (n,)))
        masses = _f64(masses, shape=(n, 3))
        x = _f64(x, shape=(n, 5))
        out = {k: np.zeros(n) for k in api.KDATA_FIELDS}
        soa = api.pnjl_kdata_soa(**{k: _dp(v) for k, v in out.items()})
        rc = self._lib.pnjl_kdata_batch(self._ctx, n, int(p_num), float(p_max), _dp(T), _dp(mu_u), _dp(mu_s),
                                        _dp(masses), _dp(x), C.byref(soa))
        self._check(rc, "pnjl_kdata_batch")
        return out

    # -- implicit derivatives of solved states ----------------------------------------------
    def derivs(self, x, T, mu, xi) -> dict:
        """Implicit derivatives (ThermoDerivatives.jl) at solved states x [n,5], host arrays:
        dx/dtheta, dM/dtheta, s, n_B and their total derivatives, P and eps with theirs, and
        the bulk-viscosity combinations; theta = (T, mu) with every mu_f moved together.
        Returns {field: [n] or [n, width]} over _capi.DERIV_FIELDS."""
        n, T, mu_u, mu_d, mu_s, xi = self._point_arrays(T, mu, xi)
        x = _f64(x, shape=(n, 5))
        out = {k: np.zeros((n, w)) if w > 1 else np.zeros(n) for k, w in api.DERIV_FIELDS}
        soa = api.pnjl_deriv_soa(**{k: _dp(v) for k, v in out.items()})
        rc = self._lib.pnjl_derivs_batch(self._ctx, n, _dp(x), _dp(T), _dp(mu_u), _dp(mu_d), _dp(mu_s), _dp(xi),
                                         C.byref(soa))
        self._check(rc, "pnjl_derivs_batch")
        return out

    def derivs_device(self, n: int, d_x: int, d_T: int, d_mu_u: int, d_mu_d: int, d_mu_s: int, d_xi: int,
                      d_out: dict):
        """Asynchronous implicit derivatives on device pointers (integers); d_out maps
        DERIV_FIELDS names to device pointers (missing ones are skipped)."""
        soa = api.pnjl_deriv_soa(**{k: C.cast(C.c_void_p(v), api.dp) for k, v in d_out.items()})
        cast = lambda p: C.cast(C.c_void_p(p), api.dp)  # noqa: E731
        rc = self._lib.pnjl_derivs_batch_device(self._ctx, n, cast(d_x), cast(d_T), cast(d_mu_u), cast(d_mu_d),
                                                cast(d_mu_s), cast(d_xi), C.byref(soa))
        self._check(rc, "pnjl_derivs_batch_device")

    def kdata_device(self, n: int, d_T: int, d_mu_u: int, d_mu_s: int, d_masses: int, d_x: int, d_out: dict, *,
                     p_num: int = 64, p_max: float = 10.0):
        """Asynchronous build_K_data on device pointers (integers), e.g. a solve's outputs;
        d_out maps KDATA_FIELDS names to device pointers (missing ones are skipped)."""
        soa = api.pnjl_kdata_soa(**{k: C.cast(C.c_void_p(v), api.dp) for k, v in d_out.items()})
        cast = lambda p: C.cast(C.c_void_p(p), api.dp)  # noqa: E731
        rc = self._lib.pnjl_kdata_batch_device(self._ctx, n, int(p_num), float(p_max), cast(d_T), cast(d_mu_u),
                                               cast(d_mu_s), cast(d_masses), cast(d_x), C.byref(soa))
        self._check(rc, "pnjl_kdata_batch_device")

    # -- misc ------------------------------------------------------------------------------
    def stream(self) -> int:
        return int(self._lib.pnjl_stream(self._ctx) or 0)

    def synchronize(self):
        self._check(self._lib.pnjl_synchronize(self._ctx), "pnjl_synchronize")

    def stats(self, kernel: int | None = None) -> dict:
        """Counters of the last solve; kernel 0 / 1: the per-point / task kernel of a mixed
        per-point solve alone (pnjl_get_kernel_stats)."""
        st = api.pnjl_stats()
        if kernel is None:
            self._check(self._lib.pnjl_get_stats(self._ctx, C.byref(st)), "pnjl_get_stats")
        else:
            self._check(self._lib.pnjl_get_kernel_stats(self._ctx, int(kernel), C.byref(st)), "pnjl_get_kernel_stats")
        return {k: getattr(st, k) for k, _ in api.pnjl_stats._fields_}

    def set_wait_limits(self, ready_polls: int, verdict_polls: int):
        """Bounds of the fused kernel's waits on flags of the same launch (pnjl_set_wait_limits)."""
        self._check(self._lib.pnjl_set_wait_limits(self._ctx, int(ready_polls), int(verdict_polls)),
                    "pnjl_set_wait_limits")

    def wait_limits(self) -> tuple[int, int]:
        r, v = C.c_uint32(), C.c_uint32()
        self._check(self._lib.pnjl_get_wait_limits(self._ctx, C.byref(r), C.byref(v)), "pnjl_get_wait_limits")
        return int(r.value), int(v.value)

    def sm_count(self) -> int:
        return int(self._lib.pnjl_device_sm_count(self._ctx))

    def probe_peak(self, kind: str) -> float:
        """Measured pipe throughput: "fp64" / "fp32" FLOP/s (FMA = 2) or "sfu" ex2 ops/s."""
        v = C.c_double()
        k = {"fp64": 0, "fp32": 1, "sfu": 2, "fp64_one_lane": 3}[kind]
        self._check(self._lib.pnjl_probe_peak(self._ctx, k, C.byref(v)), "pnjl_probe_peak")
        return float(v.value)

    def f64_math(self, fn: str, x) -> np.ndarray:
        """Element-wise function on the device (pnjl_f64_math): "exp", "rcp", "rsqrt" (the FP64
        certification pass's own), "exp_lib", "rcp_lib", "rsqrt_lib" (the library's), or
        "ff_exp", "ff_log" (the float-float passes', on x rounded to a float pair)."""
        k = {"exp": 0, "rcp": 1, "rsqrt": 2, "exp_lib": 3, "rcp_lib": 4, "rsqrt_lib": 5, "ff_exp": 6, "ff_log": 7}[fn]
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        dp = C.POINTER(C.c_double)
        self._check(self._lib.pnjl_f64_math(self._ctx, k, x.size, x.ctypes.data_as(dp), y.ctypes.data_as(dp)),
                    "pnjl_f64_math")
        return y

    def set_tuning(self, lanes_per_point: int, blocks_per_sm: int = 0, pipeline_chunks: int | None = None,
                   cert_warps: int | None = None):
        self._check(self._lib.pnjl_set_tuning(self._ctx, int(lanes_per_point), int(blocks_per_sm)),
                    "pnjl_set_tuning")
        if pipeline_chunks is not None:
            self._check(self._lib.pnjl_set_pipeline(self._ctx, int(pipeline_chunks)), "pnjl_set_pipeline")
        if cert_warps is not None:
            self._check(self._lib.pnjl_set_cert_warps(self._ctx, int(cert_warps)), "pnjl_set_cert_warps")

    def tuning(self) -> dict:
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        self._check(self._lib.pnjl_get_tuning(self._ctx, C.byref(a), C.byref(b), C.byref(c)), "pnjl_get_tuning")
        k = C.c_int32()
        self._check(self._lib.pnjl_get_cert_warps(self._ctx, C.byref(k)), "pnjl_get_cert_warps")
        return {"lanes_per_point": a.value, "blocks_per_sm": b.value, "pipeline_chunks": c.value,
                "cert_warps": k.value}

    def autotune(self, n: int, d_T: int, d_mu_u: int, d_mu_d: int, d_mu_s: int, d_xi: int, d_out: dict, *,
                 seed_table=None, seed_table_hot=None, hot_T_MeV: float = 300.0, opts: SolveOptions | None = None,
                 learned: bool = False, reps: int = 2):
        """pnjl_autotune on a representative device batch: tries the launch shapes, keeps the
        fastest on this context; returns (best, [all tried]) as dicts."""
        opts = opts or SolveOptions()
        st = None if seed_table is None else _f64(seed_table).reshape(-1, 5)
        sth = None if seed_table_hot is None else _f64(seed_table_hot).reshape(-1, 5)
        o = self._opts_struct(opts, st, sth, hot_T_MeV, False, None)
        soa = api.pnjl_result_soa()
        for k, v in d_out.items():
            ptr_t = dict(iterations=api.i32p, chosen_seed=api.i32p, status=api.i32p, converged=api.u8p).get(k, api.dp)
            setattr(soa, k, C.cast(C.c_void_p(v), ptr_t))
        cast = lambda p: C.cast(C.c_void_p(p), api.dp)  # noqa: E731
        best = api.pnjl_tuning()
        tried = (api.pnjl_tuning * 64)()
        nt = C.c_int32()
        rc = self._lib.pnjl_autotune(self._ctx, n, cast(d_T), cast(d_mu_u), cast(d_mu_d), cast(d_mu_s), cast(d_xi),
                                     C.byref(o), C.byref(soa), int(learned), int(reps), C.byref(best), tried, 64,
                                     C.byref(nt))
        self._check(rc, "pnjl_autotune")
        as_dict = lambda t: {k: getattr(t, k) for k, _ in api.pnjl_tuning._fields_}  # noqa: E731
        return as_dict(best), [as_dict(tried[i]) for i in range(min(nt.value, 64))]


class SolvePlan:
    """Several batched solves -- each with its own quadrature order, device inputs, outputs and
    options -- captured into one CUDA graph and replayed with one launch (pnjl_plan_*).

    Typical use: the same (T, mu, xi) grid at p = 64, 128 and 256 nodes (a quadrature
    convergence study), or slices of a scan with different orders, in one launch."""

    def __init__(self, engine: GapEngine):
        self.engine = engine
        self._lib = engine._lib
        h = C.c_void_p()
        engine._check(self._lib.pnjl_plan_create(engine._ctx, C.byref(h)), "pnjl_plan_create")
        self._h = h
        self.segments = 0

    def add(self, p_num: int, t_num: int, n: int, d_T: int, d_mu_u: int, d_mu_d: int, d_mu_s: int, d_xi: int,
            d_out: dict, *, seed_table=None, seed_table_hot=None, hot_T_MeV: float = 300.0,
            opts: SolveOptions | None = None, learned: bool = False, p_max: float = 10.0, d_point_seeds: int = 0):
        """Add a segment (device pointers as integers; d_out maps result fields to device pointers).
        Host tables are copied now."""
        opts = opts or SolveOptions()
        st = None if seed_table is None else _f64(seed_table).reshape(-1, 5)
        sth = None if seed_table_hot is None else _f64(seed_table_hot).reshape(-1, 5)
        ps = None if learned else (d_point_seeds or None)
        o = GapEngine._opts_struct(opts, st, sth, hot_T_MeV, ps is not None, ps)
        soa = api.pnjl_result_soa()
        for k, v in d_out.items():
            ptr_t = dict(iterations=api.i32p, chosen_seed=api.i32p, status=api.i32p, converged=api.u8p).get(k, api.dp)
            setattr(soa, k, C.cast(C.c_void_p(v), ptr_t))
        cast = lambda p: C.cast(C.c_void_p(p), api.dp)  # noqa: E731
        rc = self._lib.pnjl_plan_add(self._h, int(p_num), int(t_num), float(p_max), int(n), cast(d_T), cast(d_mu_u),
                                     cast(d_mu_d), cast(d_mu_s), cast(d_xi), C.byref(o), int(bool(learned)),
                                     C.byref(soa))
        self.engine._check(rc, "pnjl_plan_add")
        self.segments += 1
        return self.segments - 1

    def finalize(self):
        self.engine._check(self._lib.pnjl_plan_finalize(self._h), "pnjl_plan_finalize")

    def launch(self):
        """One graph launch on the engine's stream (asynchronous)."""
        self.engine._check(self._lib.pnjl_plan_launch(self._h), "pnjl_plan_launch")

    def stats(self, segment: int = -1) -> dict:
        st = api.pnjl_stats()
        self.engine._check(self._lib.pnjl_plan_stats(self._h, int(segment), C.byref(st)), "pnjl_plan_stats")
        return {k: getattr(st, k) for k, _ in api.pnjl_stats._fields_}

    def close(self):
        if self._h:
            self._lib.pnjl_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 -- interpreter shutdown
            pass

