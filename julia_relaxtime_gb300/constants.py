"""Model constants of the PNJL parameter set (src/Constants_PNJL.jl, config/pnjl/*.toml).

``load_pnjl_config(profile)`` mirrors Constants_PNJL.jl:57-73: built-in defaults, deep-merged
with ``<config_dir>/<profile>.toml`` when that file exists (profile from the environment
variable ``PNJL_PARAM_PROFILE``, default "default").  ``PNJLParams`` holds the derived fm-unit
constants of :82-103 and converts to the C struct ``pnjl_params``.
"""
from __future__ import annotations

import copy
import os
import tomllib
import warnings
from dataclasses import dataclass

DEFAULT_CONFIG = {
    "physical": {"hbarc": 197.327, "alpha_em": 1.0 / 137.035999084},
    "model": {"N_color": 3, "N_flavor": 3, "rho0_fm3": 0.16, "Lambda_MeV": 602.3, "G_over_Lambda2": 1.835,
              "K_over_Lambda5": 12.36, "m_ud0_MeV": 5.5, "m_s0_MeV": 140.7},
    "polyakov": {"T0_MeV": 210.0, "a0": 3.51, "a1": -2.47, "a2": 15.2, "b3": -1.75, "b4": 7.555},
}

HBARC_MEV_FM = 197.327


def _deep_merge(base: dict, override: dict) -> dict:
    out = copy.deepcopy(base)
    for k, v in override.items():
        if isinstance(v, dict) and isinstance(out.get(k), dict):
            out[k] = _deep_merge(out[k], v)
        else:
            out[k] = v
    return out


def load_pnjl_config(profile: str | None = None, config_dir: str | None = None) -> dict:
    profile = profile or os.environ.get("PNJL_PARAM_PROFILE", "default")
    cfg = copy.deepcopy(DEFAULT_CONFIG)
    path = None
    if config_dir is not None:
        path = os.path.join(config_dir, f"{profile}.toml")
        if os.path.isfile(path):
            try:
                with open(path, "rb") as fh:
                    cfg = _deep_merge(cfg, tomllib.load(fh))
            except Exception as e:  # the reference warns and keeps the defaults
                warnings.warn(f"failed to parse PNJL config {path}: {e}; using built-in defaults")
        elif profile != "default":
            warnings.warn(f"PNJL config profile {profile!r} not found at {path}; using built-in defaults")
            path = None
        else:
            path = None
    return {"config": cfg, "profile": profile, "path": path}


@dataclass(frozen=True)
class PNJLParams:
    hbarc_MeV_fm: float
    Lambda: float
    G: float
    K: float
    m_ud0: float
    m_s0: float
    T0: float
    a0: float
    a1: float
    a2: float
    b3: float
    N_color: float
    rho0: float

    @classmethod
    def from_config(cls, cfg: dict) -> "PNJLParams":
        hbarc = float(cfg["physical"]["hbarc"])
        m = cfg["model"]
        pk = cfg["polyakov"]
        Lam = float(m["Lambda_MeV"]) / hbarc
        return cls(
            hbarc_MeV_fm=hbarc,
            Lambda=Lam,
            G=float(m["G_over_Lambda2"]) / Lam ** 2,
            K=float(m["K_over_Lambda5"]) / Lam ** 5,
            m_ud0=float(m["m_ud0_MeV"]) / hbarc,
            m_s0=float(m["m_s0_MeV"]) / hbarc,
            T0=float(pk["T0_MeV"]) / hbarc,
            a0=float(pk["a0"]), a1=float(pk["a1"]), a2=float(pk["a2"]), b3=float(pk["b3"]),
            N_color=float(m["N_color"]),
            rho0=float(m["rho0_fm3"]),
        )

    @classmethod
    def default(cls) -> "PNJLParams":
        return cls.from_config(DEFAULT_CONFIG)

    @classmethod
    def load(cls, profile: str | None = None, config_dir: str | None = None) -> "PNJLParams":
        return cls.from_config(load_pnjl_config(profile, config_dir)["config"])

    def to_c(self):
        from ._capi import pnjl_params

        p = pnjl_params()
        for k in pnjl_params._fields_:
            setattr(p, k[0], getattr(self, k[0]))
        return p
