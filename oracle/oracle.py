"""ctypes wrapper around the CPU FP64 oracle (oracle/pnjl_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and by
bench.py's CPU-baseline leg, always as the checker.  The product package
``julia_relaxtime_gb300`` never imports this module.

The oracle restates the reference's Julia path (src/pnjl/core, src/pnjl/solver) in C;
see the header of pnjl_oracle.c for the file:line map.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "lib", "libpnjl_oracle.so")


class Params(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "hbarc_MeV_fm", "Lambda", "G", "K", "m_ud0", "m_s0", "T0",
        "a0", "a1", "a2", "b3", "N_color", "rho0")]


class Opts(C.Structure):
    _fields_ = [
        ("max_iter", C.c_int),
        ("ftol", C.c_double),
        ("xtol", C.c_double),
        ("residual_norm_max", C.c_double),
        ("phi_tol", C.c_double),
        ("omega_tie_rtol", C.c_double),
        ("trust_region_fallback", C.c_int),
        ("auto_multiseed_fallback", C.c_int),
    ]


class Result(C.Structure):
    _fields_ = [
        ("converged", C.c_int),
        ("x", C.c_double * 5),
        ("omega", C.c_double),
        ("pressure", C.c_double),
        ("rho_norm", C.c_double),
        ("entropy", C.c_double),
        ("energy", C.c_double),
        ("masses", C.c_double * 3),
        ("iterations", C.c_int),
        ("residual_norm", C.c_double),
        ("rho", C.c_double * 3),
        ("nq", C.c_double * 3),
        ("naq", C.c_double * 3),
        ("f_converged", C.c_int),
        ("phys", C.c_int),
        ("status", C.c_int),
        ("chosen_seed", C.c_int),
        ("used_fallback", C.c_int),
        ("evals", C.c_long),
    ]


class Thermo(C.Structure):
    _fields_ = [
        ("pressure", C.c_double), ("rho_norm", C.c_double), ("entropy", C.c_double), ("energy", C.c_double),
        ("rho", C.c_double * 3), ("nq", C.c_double * 3), ("naq", C.c_double * 3),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP) and return the library path."""
    src = os.path.join(_HERE, "pnjl_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        dp = C.POINTER(C.c_double)
        L.or_params_default.argtypes = [C.POINTER(Params)]
        L.or_opts_default.argtypes = [C.POINTER(Opts)]
        L.or_gauleg.argtypes = [C.c_double, C.c_double, C.c_int, dp, dp]
        L.or_build_nodes.argtypes = [C.c_int, C.c_int, C.c_double, dp, dp, dp]
        L.or_eval.argtypes = [C.POINTER(Params), C.c_int, dp, dp, dp, dp, dp, C.c_double, C.c_double, dp, dp, dp]
        L.or_thermo_eval.argtypes = [C.POINTER(Params), C.c_int, dp, dp, dp, dp, dp, C.c_double, C.c_double, C.POINTER(Thermo)]
        L.or_vacuum_integral.argtypes = [C.POINTER(Params), C.c_double]
        L.or_vacuum_integral.restype = C.c_double
        L.or_mass.argtypes = [C.POINTER(Params), dp, dp]
        L.or_solve_point.argtypes = [C.POINTER(Params), C.c_int, dp, dp, dp, C.c_double, dp, C.c_double,
                                     C.c_int, C.c_int, dp, C.POINTER(Opts), C.POINTER(Result)]
        L.or_solve_batch.argtypes = [C.POINTER(Params), C.c_int, dp, dp, dp, C.c_long, dp, dp, dp,
                                     C.c_int, C.c_int, dp, C.c_int, C.POINTER(Opts), C.POINTER(Result), C.c_int]
        L.or_multiseed_seeds.argtypes = [C.POINTER(Params), C.c_double, dp]
        L.or_builtin_seed.argtypes = [C.c_int, dp]
        L.or_max_threads.restype = C.c_int
        L.or_const_integral_term_A.argtypes = [C.POINTER(Params), C.c_double]
        L.or_const_integral_term_A.restype = C.c_double
        L.or_one_loop_A.argtypes = [C.POINTER(Params), C.c_int, dp, dp] + [C.c_double] * 5
        L.or_one_loop_A.restype = C.c_double
        L.or_kdata.argtypes = [C.POINTER(Params), C.c_int, dp, dp] + [C.c_double] * 7 + [dp]
        L.or_effective_couplings.argtypes = [C.c_double] * 4 + [dp]
        L.or_thermo_derivs.argtypes = [C.POINTER(Params), C.c_int, dp, dp, dp, dp, dp, C.c_double, C.c_double, dp]
        L.or_thermo_derivs.restype = C.c_int
        assert L.or_sizeof_result() == C.sizeof(Result), "Result layout mismatch"
        assert L.or_sizeof_opts() == C.sizeof(Opts), "Opts layout mismatch"
        assert L.or_sizeof_params() == C.sizeof(Params), "Params layout mismatch"
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def default_params() -> Params:
    p = Params()
    lib().or_params_default(C.byref(p))
    return p


def default_opts(**kw) -> Opts:
    o = Opts()
    lib().or_opts_default(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def gauleg(a: float, b: float, n: int):
    x = np.zeros(n)
    w = np.zeros(n)
    rc = lib().or_gauleg(a, b, n, _dp(x), _dp(w))
    if rc != 0:
        raise ValueError("invalid Gauss-Legendre request")
    return x, w


class Nodes:
    """Column-major p_num x t_num mesh of Integrals.jl:87-97 (flattened)."""

    def __init__(self, p_num: int, t_num: int, p_max: float = 10.0):
        n = p_num * t_num
        self.p_num, self.t_num, self.p_max = p_num, t_num, p_max
        self.p = np.zeros(n)
        self.c = np.zeros(n)
        self.w = np.zeros(n)
        rc = lib().or_build_nodes(p_num, t_num, p_max, _dp(self.p), _dp(self.c), _dp(self.w))
        if rc != 0:
            raise ValueError("invalid node request")
        self.n = n

    def args(self):
        return (self.n, _dp(self.p), _dp(self.c), _dp(self.w))


def evaluate(params: Params, nodes: Nodes, x, mu, T: float, xi: float):
    """(Omega, grad_x Omega[5], Hessian_x Omega[5,5]) at one point."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    mu = np.ascontiguousarray(mu, dtype=np.float64)
    om = np.zeros(1)
    g = np.zeros(5)
    h = np.zeros(25)
    lib().or_eval(C.byref(params), *nodes.args(), _dp(x), _dp(mu), T, xi, _dp(om), _dp(g), _dp(h))
    return float(om[0]), g, h.reshape(5, 5)


def thermo(params: Params, nodes: Nodes, x, mu, T: float, xi: float) -> dict:
    x = np.ascontiguousarray(x, dtype=np.float64)
    mu = np.ascontiguousarray(mu, dtype=np.float64)
    th = Thermo()
    lib().or_thermo_eval(C.byref(params), *nodes.args(), _dp(x), _dp(mu), T, xi, C.byref(th))
    return dict(pressure=th.pressure, rho_norm=th.rho_norm, entropy=th.entropy, energy=th.energy,
                rho=np.array(th.rho), nq=np.array(th.nq), naq=np.array(th.naq))


def vacuum_integral(params: Params, m: float) -> float:
    return lib().or_vacuum_integral(C.byref(params), m)


def mass(params: Params, x) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    m = np.zeros(3)
    lib().or_mass(C.byref(params), _dp(x), _dp(m))
    return m


def multiseed_seeds(params: Params, T_fm: float) -> np.ndarray:
    out = np.zeros(30)
    lib().or_multiseed_seeds(C.byref(params), T_fm, _dp(out))
    return out.reshape(6, 5)


BUILTIN_SEEDS = ("HADRON", "MEDIUM", "HIGH_DENSITY", "HIGH_TEMP", "VERY_HIGH_TEMP",
                 "HT_0p8", "HT_0p9", "HT_0p95", "WEAK_CHIRAL_CONF")


def builtin_seed(name: str) -> np.ndarray:
    out = np.zeros(5)
    lib().or_builtin_seed(BUILTIN_SEEDS.index(name), _dp(out))
    return out


def result_to_dict(r: Result) -> dict:
    return dict(converged=bool(r.converged), x=np.array(r.x), omega=r.omega, pressure=r.pressure,
                rho_norm=r.rho_norm, entropy=r.entropy, energy=r.energy, masses=np.array(r.masses),
                iterations=r.iterations, residual_norm=r.residual_norm, rho=np.array(r.rho),
                nq=np.array(r.nq), naq=np.array(r.naq), f_converged=bool(r.f_converged),
                phys=bool(r.phys), status=r.status, chosen_seed=r.chosen_seed,
                used_fallback=bool(r.used_fallback), evals=r.evals)


def solve_point(params: Params, nodes: Nodes, T: float, mu, xi: float, seeds, multi: bool,
                opts: Opts | None = None) -> dict:
    """mode single (multi=False: seeds is one 5-vector, auto MultiSeed fallback per opts) or
    multi (seeds is [S,5], min-Omega selection)."""
    opts = opts or default_opts()
    mu = np.ascontiguousarray(np.broadcast_to(np.asarray(mu, dtype=np.float64), (3,)))
    sd = np.ascontiguousarray(np.asarray(seeds, dtype=np.float64).reshape(-1))
    r = Result()
    lib().or_solve_point(C.byref(params), *nodes.args(), T, _dp(mu), xi, 1 if multi else 0,
                         sd.size // 5, _dp(sd), C.byref(opts), C.byref(r))
    return result_to_dict(r)


def solve_batch(params: Params, nodes: Nodes, T, mu, xi, *, seeds=None, multi=True,
                multiseed_rule=True, n_seeds=0, opts: Opts | None = None, threads: int = 0):
    """Batched solve; returns a ctypes array of Result.  mu: [n,3]."""
    opts = opts or default_opts()
    T = np.ascontiguousarray(T, dtype=np.float64)
    n = T.size
    mu = np.ascontiguousarray(np.asarray(mu, dtype=np.float64).reshape(n, 3))
    xi = np.ascontiguousarray(np.broadcast_to(np.asarray(xi, dtype=np.float64), (n,)))
    if seeds is None:
        seeds = np.zeros(5)
    sd = np.ascontiguousarray(np.asarray(seeds, dtype=np.float64).reshape(-1))
    out = (Result * n)()
    ns = n_seeds if (multi and multiseed_rule) else sd.size // 5
    lib().or_solve_batch(C.byref(params), *nodes.args(), n, _dp(T), _dp(mu), _dp(xi),
                         1 if multi else 0, ns, _dp(sd), 1 if (multi and multiseed_rule) else 0,
                         C.byref(opts), out, threads)
    return out


def polish(params: Params, nodes: Nodes, T, mu, xi, x0, *, iters: int = 4, threads: int = 0):
    """The roots x0 [n,5] converged to rounding: plain Newton (no trust region, no MultiSeed
    fallback) from x0 with ftol 1e-13 and no step test, at most `iters` steps.  Near the
    rounding floor the residual no longer falls below ftol, but the iterate stays within
    |J^-1| x rounding of the root, so x is the reference a solve at ftol 1e-10 is measured
    against.  Returns (x [n,5], omega [n], residual [n])."""
    x0 = np.ascontiguousarray(np.asarray(x0, dtype=np.float64).reshape(-1, 5))
    opts = default_opts(max_iter=iters, ftol=1e-13, xtol=0.0, trust_region_fallback=0, auto_multiseed_fallback=0)
    rs = solve_batch(params, nodes, T, mu, xi, seeds=x0, multi=False, opts=opts, threads=threads)
    x = np.array([list(r.x) for r in rs]).reshape(-1, 5)
    return x, np.array([r.omega for r in rs]), np.array([r.residual_norm for r in rs])


# build_K_data's output, in order (run_gap_transport_scan.jl:297-305, EffectiveCouplings.jl:273-278)
KDATA_FIELDS = ("A_u", "A_d", "A_s", "G_u", "G_s", "K0_plus", "K0_minus", "K123_plus", "K123_minus",
                "K4567_plus", "K4567_minus", "K8_plus", "K8_minus", "K08_plus", "K08_minus", "det_K_plus",
                "det_K_minus")


def const_integral_term_A(params: Params, m: float) -> float:
    return lib().or_const_integral_term_A(C.byref(params), m)


def one_loop_A(params: Params, p, w, m, mu, T, Phi, Phib) -> float:
    p = np.ascontiguousarray(p, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    return lib().or_one_loop_A(C.byref(params), p.size, _dp(p), _dp(w), m, mu, T, Phi, Phib)


def effective_couplings(G: float, K: float, G_u: float, G_s: float) -> dict:
    """calculate_effective_couplings (EffectiveCouplings.jl:242-279)."""
    out = np.zeros(12)
    lib().or_effective_couplings(G, K, G_u, G_s, _dp(out))
    return dict(zip(KDATA_FIELDS[5:], out.tolist()))


def kdata(params: Params, T, mu_u, mu_s, masses, x, *, p_num: int = 64, p_max: float = 10.0) -> dict:
    """build_K_data at n points: A on the p_num Gauss-Legendre nodes of [0, p_max] (the
    reference's DEFAULT_MOMENTUM_NODES: 64 on [0, 10]); masses [n,3], x [n,5] (Phi = x[:,3],
    Phibar = x[:,4]).  Returns {field: [n]} over KDATA_FIELDS."""
    p, w = gauleg(0.0, p_max, p_num)
    T = np.atleast_1d(np.asarray(T, dtype=np.float64))
    n = T.size
    mu_u = np.broadcast_to(np.asarray(mu_u, dtype=np.float64), (n,))
    mu_s = np.broadcast_to(np.asarray(mu_s, dtype=np.float64), (n,))
    masses = np.asarray(masses, dtype=np.float64).reshape(n, 3)
    x = np.asarray(x, dtype=np.float64).reshape(n, 5)
    out = np.zeros((n, len(KDATA_FIELDS)))
    row = np.zeros(len(KDATA_FIELDS))
    for i in range(n):
        lib().or_kdata(C.byref(params), p.size, _dp(p), _dp(w), T[i], mu_u[i], mu_s[i], masses[i, 0], masses[i, 2],
                       x[i, 3], x[i, 4], _dp(row))
        out[i] = row
    return {k: out[:, j].copy() for j, k in enumerate(KDATA_FIELDS)}


DERIV_FIELDS = ("dx_dT", "dx_dmu", "dM_dT", "dM_dmu", "s", "n_B", "ds_dT", "ds_dmu", "dn_dT", "dn_dmu", "pressure",
                "dP_dT", "dP_dmu", "energy", "deps_dT", "deps_dmu", "dP_deps_n", "dP_dn_eps", "v_n_sq",
                "dmuB_dT_sigma")


def thermo_derivs(params: Params, nodes: Nodes, x, mu, T: float, xi: float) -> dict:
    """Implicit derivatives of a solved state (ThermoDerivatives.jl): theta = (T, mu) with every
    mu_f moved together; see or_thermo_derivs for the fields."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    mu = np.ascontiguousarray(np.broadcast_to(np.asarray(mu, dtype=np.float64), (3,)))
    out = np.zeros(32)
    rc = lib().or_thermo_derivs(C.byref(params), *nodes.args(), _dp(x), _dp(mu), T, xi, _dp(out))
    if rc != 0:
        raise ValueError("singular Hessian")
    return dict(dx_dT=out[0:5].copy(), dx_dmu=out[5:10].copy(), dM_dT=out[10:13].copy(), dM_dmu=out[13:16].copy(),
                s=out[16], n_B=out[17], ds_dT=out[18], ds_dmu=out[19], dn_dT=out[20], dn_dmu=out[21],
                pressure=out[22], dP_dT=out[23], dP_dmu=out[24], energy=out[25], deps_dT=out[26],
                deps_dmu=out[27], dP_deps_n=out[28], dP_dn_eps=out[29], v_n_sq=out[30], dmuB_dT_sigma=out[31])


def max_threads() -> int:
    return lib().or_max_threads()
