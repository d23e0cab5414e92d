"""GB300-native PNJL gap-equation scan engine (drop-in for the gap solve of w5851/Julia_RelaxTime).

Layers:
  constants   model parameters (Constants_PNJL.jl)
  _capi       ctypes declarations of include/pnjl_cuda.h
  engine      GapEngine: one libpnjl_cuda context (one GPU, one stream)
  pnjl        the reference's Julia API mirrored: solve(FixedMu(), ...), SeedStrategy, SolverResult
  scan        run_gap_transport_scan: the batched scan driver and its CSV
"""
from .constants import HBARC_MEV_FM, PNJLParams, load_pnjl_config  # noqa: F401

__all__ = ["HBARC_MEV_FM", "PNJLParams", "load_pnjl_config"]
