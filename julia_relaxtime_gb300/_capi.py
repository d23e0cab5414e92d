"""ctypes declarations of include/pnjl_cuda.h (the C ABI of libpnjl_cuda).

This module only loads the in-tree library; it never falls back to anything else.  When
the library is missing or cannot be loaded, :func:`lib` raises ``CudaLibraryError``.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libpnjl_cuda.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "pnjl_cuda.h")

PNJL_OK = 0
PNJL_ERR_INVALID_ARGUMENT = 1
PNJL_ERR_CUDA = 2
PNJL_ERR_NO_NODES = 3
PNJL_ERR_OUT_OF_MEMORY = 4
PNJL_ERR_NOT_TRAINED = 5
PNJL_ERR_TIMEOUT = 6
PNJL_ERR_TOO_LARGE = 7
PNJL_NOALLOC_MAX_TASKS = 32768

PNJL_POINT_CONVERGED = 0
PNJL_POINT_NOT_CONVERGED = 1
PNJL_POINT_EXCEPTION = 2
PNJL_POINT_ALL_SEEDS_FAILED = 3
PNJL_POINT_INVALID_INPUT = 4

PNJL_SEEDS_TABLE = 0
PNJL_SEEDS_PER_POINT = 1

PNJL_PREC_FP64 = 0
PNJL_PREC_MIXED = 1
PNJL_PREC_FF_RESIDUAL = 2  # pnjl_eval_batch only
PNJL_PREC_FP64_CERT = 3  # pnjl_eval_batch only
PNJL_PREC_FP32_NEWTON = 4  # pnjl_eval_batch only

dp = C.POINTER(C.c_double)
i32p = C.POINTER(C.c_int32)
u8p = C.POINTER(C.c_uint8)


class CudaLibraryError(RuntimeError):
    """libpnjl_cuda is missing, failed to load, or returned an error code."""


class pnjl_params(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "hbarc_MeV_fm", "Lambda", "G", "K", "m_ud0", "m_s0", "T0", "a0", "a1", "a2", "b3", "N_color", "rho0")]


class pnjl_solve_opts(C.Structure):
    _fields_ = [
        ("seed_mode", C.c_int32),
        ("n_seeds", C.c_int32),
        ("seed_table", dp),
        ("seed_table_hot", dp),
        ("hot_T_MeV", C.c_double),
        ("point_seeds", dp),
        ("max_iter", C.c_int32),
        ("ftol", C.c_double),
        ("xtol", C.c_double),
        ("residual_norm_max", C.c_double),
        ("phi_tol", C.c_double),
        ("omega_tie_rtol", C.c_double),
        ("trust_region_fallback", C.c_int32),
        ("auto_multiseed_fallback", C.c_int32),
        ("precision", C.c_int32),
        ("verify_seeds", C.c_int32),
        ("verify_T_max_MeV", C.c_double),
        ("verify_max_step", C.c_double),
        ("verify_map", u8p),
        ("verify_map_dims", C.c_int32 * 3),
        ("verify_map_lo", C.c_double * 3),
        ("verify_map_hi", C.c_double * 3),
    ]


class pnjl_result_soa(C.Structure):
    _fields_ = [
        ("x", dp), ("omega", dp), ("pressure", dp), ("rho_norm", dp), ("entropy", dp), ("energy", dp),
        ("masses", dp), ("rho", dp), ("n_q", dp), ("n_aq", dp), ("residual_norm", dp),
        ("iterations", i32p), ("chosen_seed", i32p), ("status", i32p), ("converged", u8p),
    ]


KDATA_FIELDS = ("A_u", "A_d", "A_s", "G_u", "G_s", "K0_plus", "K0_minus", "K123_plus", "K123_minus",
                "K4567_plus", "K4567_minus", "K8_plus", "K8_minus", "K08_plus", "K08_minus", "det_K_plus",
                "det_K_minus")


class pnjl_kdata_soa(C.Structure):
    _fields_ = [(k, dp) for k in KDATA_FIELDS]


# fields of pnjl_deriv_soa with their widths per point
DERIV_FIELDS = (("dx_dT", 5), ("dx_dmu", 5), ("dM_dT", 3), ("dM_dmu", 3), ("s", 1), ("n_B", 1), ("ds_dT", 1),
                ("ds_dmu", 1), ("dn_dT", 1), ("dn_dmu", 1), ("pressure", 1), ("dP_dT", 1), ("dP_dmu", 1),
                ("energy", 1), ("deps_dT", 1), ("deps_dmu", 1), ("dP_deps_n", 1), ("dP_dn_eps", 1),
                ("v_n_sq", 1), ("dmuB_dT_sigma", 1))


class pnjl_deriv_soa(C.Structure):
    _fields_ = [(k, dp) for k, _ in DERIV_FIELDS]


class pnjl_stats(C.Structure):
    _fields_ = [
        ("points", C.c_int64), ("passes_fp64", C.c_int64), ("passes_fp32", C.c_int64),
        ("node_evals_fp64", C.c_int64), ("node_evals_fp64_newton", C.c_int64), ("node_evals_fp64_thermo", C.c_int64),
        ("node_evals_fp64_grad", C.c_int64), ("node_evals_fp64_grad_thermo", C.c_int64),
        ("node_evals_fp32", C.c_int64), ("seeds_run", C.c_int64), ("trust_region_runs", C.c_int64),
        ("multiseed_fallbacks", C.c_int64), ("kernel_launches", C.c_int64), ("last_kernel_ms", C.c_double),
        ("fp64_rescues", C.c_int64), ("node_evals_fp32_thermo", C.c_int64), ("pruned_candidates", C.c_int64),
        ("node_evals_ff", C.c_int64), ("node_evals_ff_thermo", C.c_int64), ("device_wait_timeouts", C.c_int64),
        ("node_evals_ff_grad_thermo", C.c_int64),
    ]


class pnjl_tuning(C.Structure):
    _fields_ = [("lanes_per_point", C.c_int32), ("blocks_per_sm", C.c_int32), ("pipeline_chunks", C.c_int32),
                ("cert_warps", C.c_int32), ("ms", C.c_double)]


# name -> (restype, argtypes); every function declared in include/pnjl_cuda.h
SIGNATURES = {
    "pnjl_params_default": (C.c_int, [C.POINTER(pnjl_params)]),
    "pnjl_init": (C.c_int, [C.POINTER(pnjl_params), C.c_int, C.POINTER(C.c_void_p)]),
    "pnjl_destroy": (C.c_int, [C.c_void_p]),
    "pnjl_last_error": (C.c_char_p, [C.c_void_p]),
    "pnjl_set_nodes": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_double]),
    "pnjl_get_nodes": (C.c_int, [C.c_void_p, dp, dp, dp]),
    "pnjl_eval_batch": (C.c_int, [C.c_void_p, C.c_int64, dp, dp, dp, dp, dp, dp, C.c_int32, dp, dp, dp]),
    "pnjl_thermo_batch": (C.c_int, [C.c_void_p, C.c_int64, dp, dp, dp, dp, dp, dp, C.POINTER(pnjl_result_soa)]),
    "pnjl_solve_batch": (C.c_int, [C.c_void_p, C.c_int64, dp, dp, dp, dp, dp,
                                   C.POINTER(pnjl_solve_opts), C.POINTER(pnjl_result_soa)]),
    "pnjl_solve_batch_device": (C.c_int, [C.c_void_p, C.c_int64, dp, dp, dp, dp, dp,
                                          C.POINTER(pnjl_solve_opts), C.POINTER(pnjl_result_soa)]),
    "pnjl_stream": (C.c_void_p, [C.c_void_p]),
    "pnjl_synchronize": (C.c_int, [C.c_void_p]),
    "pnjl_get_stats": (C.c_int, [C.c_void_p, C.POINTER(pnjl_stats)]),
    "pnjl_get_kernel_stats": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(pnjl_stats)]),
    "pnjl_device_sm_count": (C.c_int, [C.c_void_p]),
    "pnjl_set_tuning": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "pnjl_set_pipeline": (C.c_int, [C.c_void_p, C.c_int32]),
    "pnjl_set_cert_warps": (C.c_int, [C.c_void_p, C.c_int32]),
    "pnjl_get_cert_warps": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "pnjl_autotune": (C.c_int, [C.c_void_p, C.c_int64, dp, dp, dp, dp, dp, C.POINTER(pnjl_solve_opts),
                                C.POINTER(pnjl_result_soa), C.c_int32, C.c_int32, C.POINTER(pnjl_tuning),
                                C.POINTER(pnjl_tuning), C.c_int32, C.POINTER(C.c_int32)]),
    "pnjl_set_wait_limits": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32]),
    "pnjl_get_wait_limits": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "pnjl_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "pnjl_probe_peak": (C.c_int, [C.c_void_p, C.c_int32, dp]),
    "pnjl_f64_math": (C.c_int, [C.c_void_p, C.c_int32, C.c_int64, dp, dp]),
    "pnjl_mlp_param_count": (C.c_int, []),
    "pnjl_mlp_init": (C.c_int, [C.c_void_p, C.c_uint64]),
    "pnjl_mlp_set_scaling": (C.c_int, [C.c_void_p, dp, dp, dp, dp]),
    "pnjl_mlp_train": (C.c_int, [C.c_void_p, C.c_int64, dp, dp, dp, dp, C.c_int32, C.c_int32, C.c_double,
                                 C.c_uint64, dp]),
    "pnjl_mlp_loss_grad": (C.c_int, [C.c_void_p, C.c_int64, dp, dp, dp, dp, dp, C.POINTER(C.c_float)]),
    "pnjl_mlp_infer": (C.c_int, [C.c_void_p, C.c_int64, dp, dp, dp, dp]),
    "pnjl_mlp_infer_device": (C.c_int, [C.c_void_p, C.c_int64, dp, dp, dp, dp]),
    "pnjl_mlp_get_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_int64]),
    "pnjl_mlp_set_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float), C.c_int64]),
    "pnjl_solve_batch_learned_device": (C.c_int, [C.c_void_p, C.c_int64, dp, dp, dp, dp, dp,
                                                  C.POINTER(pnjl_solve_opts), C.POINTER(pnjl_result_soa)]),
    "pnjl_solve_batch_learned": (C.c_int, [C.c_void_p, C.c_int64, dp, dp, dp, dp, dp,
                                           C.POINTER(pnjl_solve_opts), C.POINTER(pnjl_result_soa)]),
    "pnjl_plan_create": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "pnjl_plan_add": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_double, C.c_int64, dp, dp, dp, dp, dp,
                                C.POINTER(pnjl_solve_opts), C.c_int32, C.POINTER(pnjl_result_soa)]),
    "pnjl_plan_finalize": (C.c_int, [C.c_void_p]),
    "pnjl_plan_launch": (C.c_int, [C.c_void_p]),
    "pnjl_plan_stats": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(pnjl_stats)]),
    "pnjl_plan_destroy": (C.c_int, [C.c_void_p]),
    "pnjl_kdata_batch": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_double, dp, dp, dp, dp, dp,
                                   C.POINTER(pnjl_kdata_soa)]),
    "pnjl_kdata_batch_device": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_double, dp, dp, dp, dp, dp,
                                          C.POINTER(pnjl_kdata_soa)]),
    "pnjl_derivs_batch": (C.c_int, [C.c_void_p, C.c_int64, dp, dp, dp, dp, dp, dp, C.POINTER(pnjl_deriv_soa)]),
    "pnjl_derivs_batch_device": (C.c_int, [C.c_void_p, C.c_int64, dp, dp, dp, dp, dp, dp,
                                           C.POINTER(pnjl_deriv_soa)]),
    "pnjl_solve_batch_noalloc": (C.c_int, [C.POINTER(pnjl_params), C.c_int32, C.c_int32, C.c_double, C.c_int64,
                                           dp, dp, dp, dp, dp, C.POINTER(pnjl_solve_opts),
                                           C.POINTER(pnjl_result_soa), C.c_void_p]),
}

_lib = None


def lib():
    """Load libpnjl_cuda.so from the package tree (built by julia_relaxtime_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise CudaLibraryError(
            f"{LIB_PATH} is missing: build it with `python -m julia_relaxtime_gb300.build` "
            "(there is no CPU fallback)")
    try:
        L = C.CDLL(LIB_PATH)
    except OSError as e:  # pragma: no cover - depends on the machine
        raise CudaLibraryError(f"cannot load {LIB_PATH}: {e}") from e
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def declared_functions() -> list[str]:
    """Names of the functions declared in include/pnjl_cuda.h (parsed from the header)."""
    import re

    with open(HEADER) as fh:
        text = fh.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pnjl_[a-z0-9_]+)\s*\(", text)))


def check(ctx, rc: int, what: str):
    if rc != PNJL_OK:
        msg = lib().pnjl_last_error(ctx)
        msg = msg.decode() if msg else ""
        raise CudaLibraryError(f"{what} failed with code {rc}: {msg}")
