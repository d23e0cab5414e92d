// pnjl_host_common.h -- host helpers shared by the C-ABI translation units: the
// Gauss-Legendre rule, the separable node tables and the option checks.  Nothing here
// allocates memory.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#include "pnjl_f64.cuh"
#include "pnjl_ff.cuh"
#include "pnjl_kernels.h"

namespace pnjl {

// Gauss-Legendre rule on [a, b] into x[n], w[n] (ascending): Newton's method on the
// Legendre polynomial P_n evaluated by its three-term recurrence (in long double), started
// from cos(pi (k + 3/4) / (n + 1/2)); weights 2 / ((1 - x^2) P_n'(x)^2).  Same published
// rule the reference obtains from FastGaussQuadrature.gausslegendre
// (src/integration/GaussLegendre.jl:33-42, :94-119).
inline void gauss_legendre_into(int n, double a, double b, double *x, double *w) {
    const int half = (n + 1) / 2;
    for (int k = 0; k < half; ++k) {
        long double z = std::cos(M_PI * (k + 0.75) / (n + 0.5));
        long double p0 = 1.0L, p1 = z, dp = 1.0L;
        for (int iter = 0; iter < 64; ++iter) {
            p0 = 1.0L;
            p1 = z;
            for (int j = 2; j <= n; ++j) {
                long double p2 = ((2.0L * j - 1.0L) * z * p1 - (j - 1.0L) * p0) / j;
                p0 = p1;
                p1 = p2;
            }
            if (n == 1) { p1 = z; p0 = 1.0L; }
            dp = n * (z * p1 - p0) / (z * z - 1.0L);
            long double dz = p1 / dp;
            z -= dz;
            if (std::fabs((double)dz) < 1e-19) break;
        }
        p0 = 1.0L;
        p1 = z;
        for (int j = 2; j <= n; ++j) {
            long double p2 = ((2.0L * j - 1.0L) * z * p1 - (j - 1.0L) * p0) / j;
            p0 = p1;
            p1 = p2;
        }
        if (n == 1) { p1 = z; p0 = 1.0L; }
        dp = n * (z * p1 - p0) / (z * z - 1.0L);
        const double wt = (double)(2.0L / ((1.0L - z * z) * dp * dp));
        x[k] = -(double)z;
        x[n - 1 - k] = (double)z;
        w[k] = wt;
        w[n - 1 - k] = wt;
        if (2 * k + 1 == n) x[k] = 0.0;
    }
    const double scale = (b - a) / 2.0, shift = (b + a) / 2.0;
    for (int i = 0; i < n; ++i) {
        x[i] = scale * x[i] + shift;
        w[i] = scale * w[i];
    }
}

static constexpr int kMaxPNodes = 512;
static constexpr int kMaxTNodes = 64;

// Separable device tables p2[p] | A[p] = w_p p^2/(2 pi)^2 | c2[t] | B[t] = 2 w_c
// (2 (p + t) values) from the p rule on [0, p_max] and the cos(theta) rule on [0, 1].
inline void separable_tables(int p_num, int t_num, const double *xp, const double *wp, const double *xc,
                             const double *wc, double *h, float *hf, float *hl = nullptr) {
    const double fourpi2 = (2.0 * M_PI) * (2.0 * M_PI);
    for (int ip = 0; ip < p_num; ++ip) {
        h[ip] = xp[ip] * xp[ip];
        h[p_num + ip] = wp[ip] * (xp[ip] * xp[ip]) / fourpi2;
    }
    for (int it = 0; it < t_num; ++it) {
        h[2 * p_num + it] = xc[it] * xc[it];
        h[2 * p_num + t_num + it] = 2.0 * wc[it];
    }
    const int m = 2 * (p_num + t_num);
    for (int i = 0; i < m; ++i) hf[i] = (float)h[i];
    if (hl)  // float-float low parts: h = hf + hl to ~2^-48
        for (int i = 0; i < m; ++i) hl[i] = (float)(h[i] - (double)hf[i]);
}

// Function tables (pnjl_ff.cuh, pnjl_f64.cuh), from long-double exp / log: e^k for
// k = -kExpMaxN..kExpMaxN and e^(j/256) for j = 0..255, ln c_j and 1/c_j for
// c_j = 1 + (2j + 1)/256, j = 0..127, each as a (hi, lo) float pair; then 2^(j/256),
// j = 0..255, as doubles.
inline void ff_pair_into(long double v, float *out) {
    const float h = (float)v;
    out[0] = h;
    out[1] = (float)(v - (long double)h);
}
inline void ff_exp_tables(float *out) {
    for (int k = -kExpMaxN; k <= kExpMaxN; ++k) ff_pair_into(expl((long double)k), out + 2 * (k + kExpMaxN));
    for (int j = 0; j < kExpFracN; ++j) ff_pair_into(expl((long double)j / 256.0L), out + kExpFracOff + 2 * j);
    for (int j = 0; j < kLogN; ++j) {
        const long double c = 1.0L + (2.0L * j + 1.0L) / 256.0L;
        ff_pair_into(logl(c), out + kLogOff + 2 * j);
        ff_pair_into(1.0L / c, out + kLogOff + 2 * kLogN + 2 * j);
    }
    for (int j = 0; j < kExp64N; ++j) {
        const double v = (double)exp2l((long double)j / (long double)kExp64N);
        std::memcpy(out + kExp64Offset + 2 * j, &v, sizeof v);
    }
}

// Checks of pnjl_solve_opts; returns PNJL_OK or PNJL_ERR_INVALID_ARGUMENT and a message.
inline int validate_opts(const pnjl_solve_opts *o, const char **msg) {
    *msg = "";
    if (!o) { *msg = "opts is NULL"; return PNJL_ERR_INVALID_ARGUMENT; }
    if (o->seed_mode != PNJL_SEEDS_TABLE && o->seed_mode != PNJL_SEEDS_PER_POINT) {
        *msg = "unknown seed_mode";
        return PNJL_ERR_INVALID_ARGUMENT;
    }
    const bool need_table = o->seed_mode == PNJL_SEEDS_TABLE || o->auto_multiseed_fallback;
    if (need_table && (o->n_seeds < 1 || o->n_seeds > 16 || !o->seed_table)) {
        *msg = "seed table must have 1..16 rows";
        return PNJL_ERR_INVALID_ARGUMENT;
    }
    if (o->seed_mode == PNJL_SEEDS_PER_POINT && !o->point_seeds) {
        *msg = "point_seeds is NULL";
        return PNJL_ERR_INVALID_ARGUMENT;
    }
    if (o->max_iter < 0 || o->max_iter > 100000) { *msg = "max_iter out of range"; return PNJL_ERR_INVALID_ARGUMENT; }
    if (!(o->ftol > 0) || !(o->xtol >= 0) || !(o->residual_norm_max > 0) || !(o->phi_tol >= 0) ||
        !(o->omega_tie_rtol >= 0)) {
        *msg = "tolerances must be positive";
        return PNJL_ERR_INVALID_ARGUMENT;
    }
    if (o->verify_seeds < 0 || (o->verify_seeds > 0 && (!o->seed_table || o->verify_seeds > o->n_seeds))) {
        *msg = "verify_seeds must be 0..n_seeds (rows of the seed table)";
        return PNJL_ERR_INVALID_ARGUMENT;
    }
    if (o->verify_map) {
        int64_t cells = 1;
        for (int k = 0; k < 3; ++k) {
            if (o->verify_map_dims[k] < 1 || !(o->verify_map_hi[k] > o->verify_map_lo[k])) {
                *msg = "verify_map: dims must be >= 1 and lo < hi";
                return PNJL_ERR_INVALID_ARGUMENT;
            }
            cells *= o->verify_map_dims[k];
        }
        if (cells > (int64_t(1) << 24)) { *msg = "verify_map too large"; return PNJL_ERR_INVALID_ARGUMENT; }
    }
    if (o->precision != PNJL_PREC_FP64 && o->precision != PNJL_PREC_MIXED) {
        *msg = "unknown precision";
        return PNJL_ERR_INVALID_ARGUMENT;
    }
    return PNJL_OK;
}

inline void fill_solve_opts(const pnjl_solve_opts *o, SolveOpts &d) {
    d.max_iter = o->max_iter;
    d.ftol = o->ftol;
    d.xtol = o->xtol;
    d.residual_norm_max = o->residual_norm_max;
    d.phi_tol = o->phi_tol;
    d.omega_tie_rtol = o->omega_tie_rtol;
    d.trust_region_fallback = o->trust_region_fallback;
    d.auto_multiseed_fallback = o->auto_multiseed_fallback;
    d.verify_seeds = o->seed_mode == PNJL_SEEDS_PER_POINT ? o->verify_seeds : 0;
    d.verify_T_max_MeV = o->verify_T_max_MeV;
    d.verify_max_step = o->verify_max_step;
    d.vmap = nullptr;  // set by the caller to the device copy of o->verify_map
    d.ready_polls = kReadyPollsDefault;
    d.verdict_polls = kVerdictPollsDefault;
    for (int k = 0; k < 3; ++k) {
        d.vn[k] = o->verify_map ? o->verify_map_dims[k] : 0;
        d.vlo[k] = o->verify_map_lo[k];
        d.vhi[k] = o->verify_map_hi[k];
    }
}

inline int64_t verify_map_cells(const pnjl_solve_opts *o) {
    return o->verify_map ? (int64_t)o->verify_map_dims[0] * o->verify_map_dims[1] * o->verify_map_dims[2] : 0;
}

inline DevParams dev_params(const pnjl_params &p) {
    return DevParams{p.hbarc_MeV_fm, p.Lambda, p.G, p.K, p.m_ud0, p.m_s0, p.T0, p.a0, p.a1, p.a2, p.b3, p.N_color, p.rho0};
}

}  // namespace pnjl
