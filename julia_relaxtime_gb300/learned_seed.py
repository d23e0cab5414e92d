"""LearnedSeed: an MLP initial guess for the gap equations, trained on the GPU solver's own
solutions (a learned seed; the reference's seed interface is
src/pnjl/solver/SeedStrategies.jl:118).

The network (3 -> 128 -> 128 -> 128 -> 5, SiLU, BF16 weights, FP32 accumulation) lives in
the libpnjl_cuda context and is trained and evaluated by its kernels.  As a SeedStrategy it
returns one seed per point; in batches it feeds the per-point-seed solve, whose fallback is
the plain MultiSeed solve (the reference's auto_multiseed_fallback) -- so the learned seed can
only change how fast a point is solved, and the multi-seed result remains the arbiter.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, replace

import numpy as np

from . import _capi as api
from .constants import HBARC_MEV_FM
from .engine import GapEngine, SolveOptions, VerifyMap, _dp
from .pnjl import FixedMu, MultiSeed, SeedStrategy

PARAM_COUNT = None


def param_count() -> int:
    return int(api.lib().pnjl_mlp_param_count())


@dataclass
class TrainConfig:
    """The training set: a 64 x 64 x 5 solver-labelled (T 50-300 MeV, mu 0-400 MeV, xi -0.5..0.5) grid.
    mu is mu_u = mu_d; mu_s = mu_s_ratio * mu_u (the network's input is mu_u)."""
    T_MeV: tuple = (50.0, 300.0, 64)
    mu_MeV: tuple = (0.0, 400.0, 64)
    xi: tuple = (-0.5, 0.5, 5)
    epochs: int = 300
    batch: int = 1024
    lr: float = 4e-3
    seed: int = 20240611
    label_seeds: int = 6          # MultiSeed candidates used to label the grid
    label_precision: str = "mixed"
    mu_s_ratio: float = 1.0
    label_extra: tuple = ()       # seed rows appended to the label table (e.g. MEDIUM, HIGH_DENSITY)
    # verification map (coexistence_map): coexisting phases within map_gap_max (fm^-4) of the
    # minimum, label jumps above map_jump, flagged cells grown by map_grow
    map_gap_max: float = 0.01
    map_jump: float = 0.25
    map_grow: int = 0


def grid_points(cfg: TrainConfig):
    T = np.linspace(*cfg.T_MeV) / HBARC_MEV_FM
    mu = np.linspace(*cfg.mu_MeV) / HBARC_MEV_FM
    xi = np.linspace(*cfg.xi)
    Tg, mg, xg = np.meshgrid(T, mu, xi, indexing="ij")
    return Tg.ravel(), mg.ravel(), xg.ravel()


def flavour_mu(cfg: TrainConfig, mu):
    """(mu_u, mu_d, mu_s) of the label points: mu_u = mu_d = mu, mu_s = mu_s_ratio * mu."""
    mu = np.asarray(mu, dtype=np.float64)
    if cfg.mu_s_ratio == 1.0:
        return mu
    return np.stack([mu, mu, cfg.mu_s_ratio * mu], axis=1)


def box_scaling(cfg: TrainConfig):
    """(in_shift, in_scale) of the network's inputs (T, mu_u in fm^-1, xi): the training box
    mapped to [-1, 1]."""
    lo = np.array([cfg.T_MeV[0] / HBARC_MEV_FM, cfg.mu_MeV[0] / HBARC_MEV_FM, cfg.xi[0]])
    hi = np.array([cfg.T_MeV[1] / HBARC_MEV_FM, cfg.mu_MeV[1] / HBARC_MEV_FM, cfg.xi[1]])
    return 0.5 * (lo + hi), np.maximum(0.5 * (hi - lo), 1e-6)


def label_table(cfg: TrainConfig):
    from .pnjl import multiseed_table

    return multiseed_table(cfg.label_seeds, cfg.label_extra)


class LearnedSeed(SeedStrategy):
    def __init__(self, engine: GapEngine, seed: int = 1):
        self.engine = engine
        self._lib = api.lib()
        self._check(self._lib.pnjl_mlp_init(engine._ctx, int(seed)), "pnjl_mlp_init")
        self.trained = False
        self.timings = {}
        self.last_loss = None
        self.scaling = None
        self.verify_map: VerifyMap | None = None  # where the MultiSeed candidates verify a solution

    def _check(self, rc, what):
        api.check(self.engine._ctx, rc, what)

    # -- scaling -------------------------------------------------------------------------
    def set_scaling(self, in_shift, in_scale, out_shift, out_scale):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (in_shift, in_scale, out_shift, out_scale)]
        self._check(self._lib.pnjl_mlp_set_scaling(self.engine._ctx, *(_dp(a) for a in arrs)), "pnjl_mlp_set_scaling")
        self.scaling = arrs

    def default_scaling(self, targets, cfg: TrainConfig | None = None):
        """Inputs mapped to [-1, 1] over the training box (cfg; the default box without it),
        outputs standardised."""
        t = np.asarray(targets, dtype=np.float64)
        in_shift, in_scale = box_scaling(cfg or TrainConfig())
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
        extra = {}
        if self.verify_map is not None:
            extra = dict(vmap_flags=self.verify_map.flags, vmap_lo=np.array(self.verify_map.lo),
                         vmap_hi=np.array(self.verify_map.hi))
        np.savez(path, params=self.params(), in_shift=self.scaling[0], in_scale=self.scaling[1],
                 out_shift=self.scaling[2], out_scale=self.scaling[3], **extra)

    def load(self, path: str):
        d = np.load(path)
        self.set_scaling(d["in_shift"], d["in_scale"], d["out_shift"], d["out_scale"])
        self.set_params(d["params"])
        if "vmap_flags" in d:
            self.verify_map = VerifyMap(d["vmap_flags"], tuple(d["vmap_lo"]), tuple(d["vmap_hi"]))

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
        if opts.verify_map is None and self.verify_map is not None:
            opts = replace(opts, verify_map=self.verify_map)
        table, hot = (multiseed or MultiSeed()).tables()
        T_arr = np.atleast_1d(np.asarray(T, dtype=np.float64))
        return self.engine.solve(T_arr, mu, xi, seed_table=table, seed_table_hot=hot, opts=opts, learned=True)


def default_learned_opts(**kw) -> SolveOptions:
    """Options of the learned-seed solve: mixed precision, 40 iterations, and verification by
    every MultiSeed candidate where a second, metastable phase can exist -- the cells of the
    network's verification map (built from its labels, coexistence_map), or below T = 170 MeV
    without a map -- and wherever the root lies more than 0.3 (fm^-3 / Polyakov units,
    inf-norm) from the learned seed: there the multi-seed Newton judges the learned solution."""
    base = dict(iterations=40, precision="mixed", verify_seeds=-1, verify_T_max_MeV=170.0, verify_max_step=0.3)
    base.update(kw)
    return SolveOptions(**base)


def label_grid(engine: GapEngine, cfg: TrainConfig, opts: SolveOptions | None = None):
    """Solve the training grid with the multi-seed solver; returns the converged points."""
    T, mu, xi = grid_points(cfg)
    table, hot = label_table(cfg)
    opts = opts or SolveOptions(iterations=40, ftol=1e-10, precision=cfg.label_precision)
    res = engine.solve(T, flavour_mu(cfg, mu), xi, seed_table=table, seed_table_hot=hot, opts=opts)
    ok = res["converged"]
    return T[ok], mu[ok], xi[ok], res["x"][ok], res


def candidate_roots(engine: GapEngine, cfg: TrainConfig):
    """Root (NaN where not converged) and Omega of every MultiSeed candidate alone at every
    label-grid point: [N, S, 5] and [N, S]."""
    T, mu, xi = grid_points(cfg)
    mu = flavour_mu(cfg, mu)
    table, hot = label_table(cfg)
    opts = SolveOptions(iterations=40, ftol=1e-10, precision=cfg.label_precision)
    roots, omegas = [], []
    for s in range(table.shape[0]):  # each candidate alone: a one-row MultiSeed table
        r = engine.solve(T, mu, xi, seed_table=table[s:s + 1], seed_table_hot=hot[s:s + 1], opts=opts)
        roots.append(np.where(r["converged"][:, None], r["x"], np.nan))
        omegas.append(np.where(r["converged"], r["omega"], np.nan))
    return np.stack(roots, axis=1), np.stack(omegas, axis=1)


def candidates_and_labels(engine: GapEngine, cfg: TrainConfig):
    """Every MultiSeed candidate alone at every label-grid point, in ONE launch (S x N points,
    each with its candidate as the per-point seed, no fallback), and the labels the MultiSeed
    solve would give: at each point the converged candidate of lowest Omega, the earliest among
    Omegas within omega_tie_rtol (solve_multi, ImplicitSolver.jl:532-559).  Returns
    (roots [N, S, 5] NaN where not converged, omegas [N, S], labels {"x", "converged", "omega"})."""
    T, mu, xi = grid_points(cfg)
    mu3 = np.asarray(flavour_mu(cfg, mu), dtype=np.float64)
    table, hot = label_table(cfg)
    S, N = table.shape[0], T.size
    hot_pt = T * HBARC_MEV_FM >= 300.0  # DefaultSeed's hot row (SeedStrategies.jl:212-220)
    seeds = np.where(hot_pt[None, :, None], hot[:, None, :], table[:, None, :]).reshape(-1, 5)
    mu_all = np.tile(mu3, S) if mu3.ndim == 1 else np.tile(mu3, (S, 1))
    opts = SolveOptions(iterations=40, ftol=1e-10, precision=cfg.label_precision, auto_multiseed_fallback=False)
    r = engine.solve(np.tile(T, S), mu_all, np.tile(xi, S), seed_table=table, seed_table_hot=hot,
                     point_seeds=seeds, opts=opts)
    conv = np.asarray(r["converged"], dtype=bool).reshape(S, N)
    x = np.asarray(r["x"]).reshape(S, N, 5)
    om = np.asarray(r["omega"]).reshape(S, N)
    roots = np.where(conv[:, :, None], x, np.nan).transpose(1, 0, 2)
    omegas = np.where(conv, om, np.nan).T
    lab_x = np.full((N, 5), np.nan)
    lab_om = np.full(N, np.nan)
    lab_ok = np.zeros(N, dtype=bool)
    tie = SolveOptions().omega_tie_rtol
    for s_ in range(S):  # seed order: a later seed replaces the kept one only when clearly lower
        better = conv[s_] & (~lab_ok | (om[s_] < lab_om - tie * np.abs(lab_om)))
        lab_x[better] = x[s_][better]
        lab_om[better] = om[s_][better]
        lab_ok |= conv[s_]
    return roots, omegas, {"x": lab_x, "converged": lab_ok, "omega": lab_om}


def coexistence_map(engine: GapEngine, cfg: TrainConfig, labels, *, distinct: float = 0.05, gap_max: float = 1.0,
                    jump: float = 0.25, grow: int = 1, roots=None) -> VerifyMap:
    """Verification map on the label grid's cells.  A grid node is flagged where two MultiSeed
    candidates converge to different physical roots (|dx|_inf > distinct) whose Omega both lie
    within gap_max (fm^-4) of the minimum -- a second phase coexists; far-off roots such as the
    deep chirally broken solution (phi_u ~ -5.3 fm^-3, Omega ~3.5 fm^-4 above the minimum at
    low T) are not a competing phase -- or where the labelled solution jumps by more than
    `jump` to a neighbour along T or mu (the first-order line or a steep crossover passes; the
    xi step of the label grid is too coarse for this test).  A cell is flagged when any of its
    8 corner nodes is, and the flagged cells grow by `grow` cells in every direction."""
    T, mu, xi = grid_points(cfg)
    nT, nm, nx = int(cfg.T_MeV[2]), int(cfg.mu_MeV[2]), int(cfg.xi[2])
    R, Om = roots if roots is not None else candidate_roots(engine, cfg)
    node = np.zeros(T.size, dtype=bool)
    with np.errstate(invalid="ignore"):
        omin = np.nanmin(np.where(np.isfinite(Om), Om, np.inf), axis=1)
        for a in range(R.shape[1]):
            for b in range(a + 1, R.shape[1]):
                d = np.abs(R[:, a] - R[:, b]).max(axis=1)  # NaN (a seed failed) compares False
                node |= (d > distinct) & (np.maximum(Om[:, a], Om[:, b]) - omin < gap_max)
    X = labels["x"].reshape(nT, nm, nx, 5)
    ok = labels["converged"].reshape(nT, nm, nx)
    node = node.reshape(nT, nm, nx)
    for ax in range(2):
        d = np.abs(np.diff(X, axis=ax)).max(axis=-1)
        both = np.logical_and(np.take(ok, range(0, X.shape[ax] - 1), axis=ax),
                              np.take(ok, range(1, X.shape[ax]), axis=ax))
        j = (d > jump) & both
        pad = [(0, 0)] * 3
        pad[ax] = (0, 1)
        node |= np.pad(j, pad)
        pad[ax] = (1, 0)
        node |= np.pad(j, pad)
    node |= ~ok  # unlabelled nodes: verify around them too
    cells = np.zeros((max(nT - 1, 1), max(nm - 1, 1), max(nx - 1, 1)), dtype=bool)
    for dT in (0, 1):
        for dm in (0, 1):
            for dx in (0, 1):
                cells |= node[dT:dT + cells.shape[0], dm:dm + cells.shape[1], dx:dx + cells.shape[2]]
    for _ in range(grow):
        g = cells.copy()
        for ax in range(3):
            sl = [slice(None)] * 3
            sl[ax] = slice(1, None)
            sr = [slice(None)] * 3
            sr[ax] = slice(None, -1)
            g[tuple(sl)] |= cells[tuple(sr)]
            g[tuple(sr)] |= cells[tuple(sl)]
        cells = g
    lo = (cfg.T_MeV[0] / HBARC_MEV_FM, cfg.mu_MeV[0] / HBARC_MEV_FM, cfg.xi[0])
    hi = (cfg.T_MeV[1] / HBARC_MEV_FM, cfg.mu_MeV[1] / HBARC_MEV_FM, cfg.xi[1])
    return VerifyMap(cells.astype(np.uint8), lo, hi)


def train_learned_seed(engine: GapEngine, cfg: TrainConfig | None = None) -> LearnedSeed:
    """Label the grid with the multi-seed solver, train the network on the labels and build its
    verification map."""
    import time

    cfg = cfg or TrainConfig()
    t0 = time.perf_counter()
    # labels and every candidate's own root (the verification map's input) from one launch
    R, Om, res = candidates_and_labels(engine, cfg)
    Tg, mug, xig = grid_points(cfg)
    ok = res["converged"]
    T, mu, xi, x = Tg[ok], mug[ok], xig[ok], res["x"][ok]
    t1 = time.perf_counter()
    ls = LearnedSeed(engine, seed=cfg.seed)
    ls.default_scaling(x, cfg)
    ls.fit(T, mu, xi, x, epochs=cfg.epochs, batch=cfg.batch, lr=cfg.lr, shuffle_seed=cfg.seed + 1)
    t2 = time.perf_counter()
    ls.verify_map = coexistence_map(engine, cfg, res, roots=(R, Om), gap_max=cfg.map_gap_max, jump=cfg.map_jump,
                                    grow=cfg.map_grow)
    ls.timings = {"labels_and_candidates_s": t1 - t0, "fit_s": t2 - t1, "map_s": time.perf_counter() - t2}
    return ls
