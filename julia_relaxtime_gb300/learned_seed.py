"""LearnedSeed: an MLP initial guess for the gap equations, trained on the GPU solver's own
solutions (the north-star "learned seed"; the reference's seed interface is
src/pnjl/solver/SeedStrategies.jl:118).

The network (3 -> 128 -> 128 -> 128 -> 5, SiLU, BF16 weights, FP32 accumulation) lives in
the libpnjl_cuda context and is trained and evaluated by its kernels.  As a SeedStrategy it
returns one seed per point; in batches it feeds the per-point-seed solve, whose fallback is
the plain MultiSeed solve (the reference's auto_multiseed_fallback) -- so the learned seed can
only change how fast a point is solved, and the multi-seed result remains the judge.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _capi as api
from .constants import HBARC_MEV_FM
from .engine import GapEngine, SolveOptions, _dp
from .pnjl import FixedMu, MultiSeed, SeedStrategy

PARAM_COUNT = None


def param_count() -> int:
    return int(api.lib().pnjl_mlp_param_count())


@dataclass
class TrainConfig:
    """Config 4 of the scan: a 64 x 64 x 5 solver-labelled (T, mu, xi) grid."""
    T_MeV: tuple = (50.0, 300.0, 64)
    mu_MeV: tuple = (0.0, 400.0, 64)
    xi: tuple = (-0.5, 0.5, 5)
    epochs: int = 400
    batch: int = 512
    lr: float = 2e-3
    seed: int = 20240611
    label_seeds: int = 6          # MultiSeed candidates used to label the grid
    label_precision: str = "mixed"


def grid_points(cfg: TrainConfig):
    T = np.linspace(*cfg.T_MeV) / HBARC_MEV_FM
    mu = np.linspace(*cfg.mu_MeV) / HBARC_MEV_FM
    xi = np.linspace(*cfg.xi)
    Tg, mg, xg = np.meshgrid(T, mu, xi, indexing="ij")
    return Tg.ravel(), mg.ravel(), xg.ravel()


class LearnedSeed(SeedStrategy):
    def __init__(self, engine: GapEngine, seed: int = 1):
        self.engine = engine
        self._lib = api.lib()
        self._check(self._lib.pnjl_mlp_init(engine._ctx, int(seed)), "pnjl_mlp_init")
        self.trained = False
        self.last_loss = None
        self.scaling = None

    def _check(self, rc, what):
        api.check(self.engine._ctx, rc, what)

    # -- scaling -------------------------------------------------------------------------
    def set_scaling(self, in_shift, in_scale, out_shift, out_scale):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (in_shift, in_scale, out_shift, out_scale)]
        self._check(self._lib.pnjl_mlp_set_scaling(self.engine._ctx, *(_dp(a) for a in arrs)), "pnjl_mlp_set_scaling")
        self.scaling = arrs

    def default_scaling(self, targets):
        t = np.asarray(targets, dtype=np.float64)
        in_shift = np.array([175.0 / HBARC_MEV_FM, 200.0 / HBARC_MEV_FM, 0.0])
        in_scale = np.array([125.0 / HBARC_MEV_FM, 200.0 / HBARC_MEV_FM, 0.5])
        out_shift = t.mean(axis=0)
        out_scale = np.maximum(t.std(axis=0), 1e-6)
        self.set_scaling(in_shift, in_scale, out_shift, out_scale)

    # -- training ------------------------------------------------------------------------
    def fit(self, T, mu, xi, targets, *, epochs=400, batch=512, lr=2e-3, shuffle_seed=7) -> float:
        T, mu, xi = (np.ascontiguousarray(a, dtype=np.float64) for a in (T, mu, xi))
        tg = np.ascontiguousarray(targets, dtype=np.float64).reshape(-1, 5)
        if self.scaling is None:
            self.default_scaling(tg)
        loss = C.c_double()
        rc = self._lib.pnjl_mlp_train(self.engine._ctx, T.size, _dp(T), _dp(mu), _dp(xi), _dp(tg), int(epochs),
                                      int(batch), float(lr), int(shuffle_seed), C.byref(loss))
        self._check(rc, "pnjl_mlp_train")
        self.trained = True
        self.last_loss = float(loss.value)
        return self.last_loss

    def loss_grad(self, T, mu, xi, targets):
        T, mu, xi = (np.ascontiguousarray(a, dtype=np.float64) for a in (T, mu, xi))
        tg = np.ascontiguousarray(targets, dtype=np.float64).reshape(-1, 5)
        g = np.zeros(param_count(), dtype=np.float32)
        loss = C.c_double()
        rc = self._lib.pnjl_mlp_loss_grad(self.engine._ctx, T.size, _dp(T), _dp(mu), _dp(xi), _dp(tg), C.byref(loss),
                                          g.ctypes.data_as(C.POINTER(C.c_float)))
        self._check(rc, "pnjl_mlp_loss_grad")
        return float(loss.value), g

    def params(self) -> np.ndarray:
        p = np.zeros(param_count(), dtype=np.float32)
        self._check(self._lib.pnjl_mlp_get_params(self.engine._ctx, p.ctypes.data_as(C.POINTER(C.c_float)), p.size),
                    "pnjl_mlp_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._check(self._lib.pnjl_mlp_set_params(self.engine._ctx, p.ctypes.data_as(C.POINTER(C.c_float)), p.size),
                    "pnjl_mlp_set_params")
        self.trained = True

    def save(self, path: str):
        np.savez(path, params=self.params(), in_shift=self.scaling[0], in_scale=self.scaling[1],
                 out_shift=self.scaling[2], out_scale=self.scaling[3])

    def load(self, path: str):
        d = np.load(path)
        self.set_scaling(d["in_shift"], d["in_scale"], d["out_shift"], d["out_scale"])
        self.set_params(d["params"])

    # -- inference -------------------------------------------------------------------------
    def seeds(self, T, mu, xi) -> np.ndarray:
        T, mu, xi = (np.ascontiguousarray(np.atleast_1d(a), dtype=np.float64) for a in (T, mu, xi))
        n = T.size
        mu = np.ascontiguousarray(np.broadcast_to(mu, (n,)))
        xi = np.ascontiguousarray(np.broadcast_to(xi, (n,)))
        out = np.zeros((n, 5))
        self._check(self._lib.pnjl_mlp_infer(self.engine._ctx, n, _dp(T), _dp(mu), _dp(xi), _dp(out)), "pnjl_mlp_infer")
        return out

    def get_seed(self, theta, mode=None):
        """SeedStrategy interface: theta = [T_fm, mu_fm(, xi)]."""
        xi = theta[2] if len(theta) > 2 else 0.0
        return self.seeds([theta[0]], [theta[1]], [xi])[0]

    def solve(self, T, mu, xi, *, opts: SolveOptions | None = None, multiseed: MultiSeed | None = None):
        """Learned seed per point (network evaluated on the device), then one Newton solve;
        MultiSeed fallback where it does not converge, verification seeds where a second
        phase can exist (opts.verify_*; default_learned_opts())."""
        opts = opts or default_learned_opts()
        table, hot = (multiseed or MultiSeed()).tables()
        T_arr = np.atleast_1d(np.asarray(T, dtype=np.float64))
        return self.engine.solve(T_arr, mu, xi, seed_table=table, seed_table_hot=hot, opts=opts, learned=True)


def default_learned_opts(**kw) -> SolveOptions:
    """Options of the learned-seed solve: mixed precision, 40 iterations, and verification by
    the first two MultiSeed candidates below T = 170 MeV or where the root lies more than 0.3
    (in fm^-3 / Polyakov units, inf-norm) from the learned seed."""
    base = dict(iterations=40, precision="mixed", verify_seeds=2, verify_T_max_MeV=170.0, verify_max_step=0.3)
    base.update(kw)
    return SolveOptions(**base)


def label_grid(engine: GapEngine, cfg: TrainConfig, opts: SolveOptions | None = None):
    """Solve the training grid with the multi-seed solver; returns the converged points."""
    T, mu, xi = grid_points(cfg)
    from .pnjl import multiseed_table

    table, hot = multiseed_table(cfg.label_seeds)
    opts = opts or SolveOptions(iterations=40, ftol=1e-10, precision=cfg.label_precision)
    res = engine.solve(T, mu, xi, seed_table=table, seed_table_hot=hot, opts=opts)
    ok = res["converged"]
    return T[ok], mu[ok], xi[ok], res["x"][ok], res


def train_learned_seed(engine: GapEngine, cfg: TrainConfig | None = None) -> LearnedSeed:
    cfg = cfg or TrainConfig()
    T, mu, xi, x, _ = label_grid(engine, cfg)
    ls = LearnedSeed(engine, seed=cfg.seed)
    ls.fit(T, mu, xi, x, epochs=cfg.epochs, batch=cfg.batch, lr=cfg.lr, shuffle_seed=cfg.seed + 1)
    return ls
