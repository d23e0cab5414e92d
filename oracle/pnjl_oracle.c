/*
 * pnjl_oracle.c -- CPU FP64 restatement of the reference's PNJL gap-equation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA library: it is
 * compiled into oracle/lib/libpnjl_oracle.so and loaded only by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg.  The product library
 * (libpnjl_cuda.so) never links, loads or calls it.
 *
 * Parity is pinned against the reference's stored scan outputs (tests/golden/,
 * written by tests/golden/make_golden.py from the reference's data/outputs files).
 *
 * How it follows the reference (file:line in w5851/Julia_RelaxTime):
 *   constants ............ src/Constants_PNJL.jl:82-103, config/pnjl/default.toml:1-21
 *   Gauss-Legendre ....... src/integration/GaussLegendre.jl:94-119,167-170
 *                          (the reference wraps FastGaussQuadrature 1.1.0; here the
 *                          published Newton-on-P_n method is restated instead)
 *   node mesh ............ src/pnjl/core/Integrals.jl:67-110
 *   vacuum term .......... src/pnjl/core/Integrals.jl:123-145
 *   log term / log sum ... src/pnjl/core/Integrals.jl:159-259
 *   mass, chi, U, Omega .. src/pnjl/core/Thermodynamics.jl:81-206
 *   thermo, densities .... src/pnjl/core/Thermodynamics.jl:215-281,
 *                          src/QuarkDistribution.jl:14-51, src/QuarkDistribution_Aniso.jl:96-120
 *   residual F = grad P .. src/pnjl/solver/Conditions.jl:72-86,205-213
 *   Newton / trust region  src/pnjl/solver/ImplicitSolver.jl:50-151 calling NLsolve 4.5.1
 *                          (:newton with the static line search, :trust_region dogleg with
 *                          autoscaling; both restated from the published methods)
 *   solve / solve_multi .. src/pnjl/solver/ImplicitSolver.jl:211-328,532-559
 *   seeds ................ src/pnjl/solver/SeedStrategies.jl:56-95,204-284
 *   implicit derivatives . src/pnjl/derivatives/ThermoDerivatives.jl:132-173,184-249,342-465
 *   K data (one-loop A,    src/relaxtime/OneLoopIntegrals.jl:507-543,
 *   effective couplings)   src/relaxtime/EffectiveCouplings.jl:56-60,112-115,242-279,
 *                          scripts/relaxtime/run_gap_transport_scan.jl:297-305
 *
 * Derivatives are taken the way the reference takes them: the reference differentiates
 * Omega with nested ForwardDiff duals (gradient for F, Jacobian of that for J).  Here a
 * second-order forward-mode "jet" (value, 5 partials, 15 Hessian entries) runs through
 * the same expression graph, which yields the same numbers up to rounding.  Thermo
 * (rho = dP/dmu, s = dP/dT) uses a first-order jet in (mu_u, mu_d, mu_s, T).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------- */
/* Parameters (fm units), same meaning as include/pnjl_cuda.h's pnjl_params  */
/* ------------------------------------------------------------------------- */
typedef struct {
    double hbarc_MeV_fm;
    double Lambda; /* fm^-1 */
    double G;      /* fm^2 */
    double K;      /* fm^5 */
    double m_ud0;  /* fm^-1 */
    double m_s0;   /* fm^-1 */
    double T0;     /* fm^-1 */
    double a0, a1, a2, b3;
    double N_color;
    double rho0;   /* fm^-3 */
} or_params;

/* Constants_PNJL.jl:82-103 with the defaults of config/pnjl/default.toml */
void or_params_default(or_params *p) {
    const double hbarc = 197.327;
    p->hbarc_MeV_fm = hbarc;
    p->Lambda = 602.3 / hbarc;
    p->m_ud0 = 5.5 / hbarc;
    p->m_s0 = 140.7 / hbarc;
    p->G = 1.835 / (p->Lambda * p->Lambda);
    p->K = 12.36 / pow(p->Lambda, 5);
    p->T0 = 210.0 / hbarc;
    p->a0 = 3.51;
    p->a1 = -2.47;
    p->a2 = 15.2;
    p->b3 = -1.75;
    p->N_color = 3.0;
    p->rho0 = 0.16;
}

/* ------------------------------------------------------------------------- */
/* Gauss-Legendre nodes (GaussLegendre.jl:94-119)                            */
/* Newton iteration on P_n(x) from the three-term recurrence, started at the */
/* Tricomi-type guess cos(pi (i - 1/4)/(n + 1/2)); weights 2/((1-x^2)P_n'^2). */
/* Nodes are returned in ascending order on [a, b].                          */
/* ------------------------------------------------------------------------- */
int or_gauleg(double a, double b, int n, double *x, double *w) {
    if (n <= 0 || !(a < b)) return -1;
    const double scale = (b - a) / 2.0, shift = (b + a) / 2.0;
    /* extended precision keeps the endpoint weights 2/((1-x^2)P'^2) accurate to ~1 ulp */
    for (int i = 0; i < (n + 1) / 2; ++i) {
        long double z = cosl(3.14159265358979323846264338327950288L * (i + 0.75L) / (n + 0.5L));
        long double pp = 0.0L;
        for (int it = 0; it < 100; ++it) {
            long double p1 = 1.0L, p2 = 0.0L;
            for (int j = 1; j <= n; ++j) {
                long double p3 = p2;
                p2 = p1;
                p1 = ((2.0L * j - 1.0L) * z * p2 - (j - 1.0L) * p3) / j;
            }
            pp = n * (z * p1 - p2) / (z * z - 1.0L);
            long double dz = p1 / pp;
            z -= dz;
            if (fabsl(dz) < 1e-19L) break;
        }
        {
            long double p1 = 1.0L, p2 = 0.0L;
            for (int j = 1; j <= n; ++j) {
                long double p3 = p2;
                p2 = p1;
                p1 = ((2.0L * j - 1.0L) * z * p2 - (j - 1.0L) * p3) / j;
            }
            pp = n * (z * p1 - p2) / (z * z - 1.0L);
        }
        double wt = (double)(2.0L / ((1.0L - z * z) * pp * pp));
        /* z is the (i+1)-th largest root: place the symmetric pair in ascending order */
        int lo = i, hi = n - 1 - i;
        x[lo] = -(double)z; x[hi] = (double)z;
        w[lo] = wt; w[hi] = wt;
        if (lo == hi) x[lo] = 0.0;
    }
    for (int i = 0; i < n; ++i) {
        x[i] = scale * x[i] + shift;
        w[i] = scale * w[i];
    }
    return 0;
}

/* Node mesh of Integrals.jl:87-97, column-major p_num x t_num (index ip + p_num*it):
 *   p_mesh[ip,it] = p_ip, c_mesh[ip,it] = cos_it,
 *   coef[ip,it] = w_p(ip) * (2 w_c(it)) * p_ip^2 / (2 pi)^2
 * momentum nodes on [0, p_max] (p_max = 10 fm^-1), cos(theta) nodes on [0, 1]. */
int or_build_nodes(int p_num, int t_num, double p_max, double *p_mesh, double *c_mesh, double *coef) {
    double *xp = malloc(sizeof(double) * p_num), *wp = malloc(sizeof(double) * p_num);
    double *xc = malloc(sizeof(double) * t_num), *wc = malloc(sizeof(double) * t_num);
    int rc = or_gauleg(0.0, p_max, p_num, xp, wp);
    if (rc == 0) rc = or_gauleg(0.0, 1.0, t_num, xc, wc);
    if (rc == 0) {
        const double fourpi2 = (2.0 * M_PI) * (2.0 * M_PI);
        for (int it = 0; it < t_num; ++it)
            for (int ip = 0; ip < p_num; ++ip) {
                int k = ip + p_num * it;
                p_mesh[k] = xp[ip];
                c_mesh[k] = xc[it];
                coef[k] = (wp[ip] * (wc[it] * 2.0)) * (xp[ip] * xp[ip]) / fourpi2;
            }
    }
    free(xp); free(wp); free(xc); free(wc);
    return rc;
}

/* ------------------------------------------------------------------------- */
/* Second-order jet in the 5 state variables x = (phi_u, phi_d, phi_s, Phi, Phibar) */
/* ------------------------------------------------------------------------- */
#define NV 5
#define NH 15
static const int HI[NH] = {0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 3, 3, 4};
static const int HJ[NH] = {0, 1, 2, 3, 4, 1, 2, 3, 4, 2, 3, 4, 3, 4, 4};

typedef struct { double v, g[NV], h[NH]; } jet;

static inline jet j_const(double c) { jet r; memset(&r, 0, sizeof r); r.v = c; return r; }
static inline jet j_var(double c, int i) { jet r = j_const(c); r.g[i] = 1.0; return r; }
static inline jet j_add(jet a, jet b) {
    jet r; r.v = a.v + b.v;
    for (int i = 0; i < NV; ++i) r.g[i] = a.g[i] + b.g[i];
    for (int k = 0; k < NH; ++k) r.h[k] = a.h[k] + b.h[k];
    return r;
}
static inline jet j_sub(jet a, jet b) {
    jet r; r.v = a.v - b.v;
    for (int i = 0; i < NV; ++i) r.g[i] = a.g[i] - b.g[i];
    for (int k = 0; k < NH; ++k) r.h[k] = a.h[k] - b.h[k];
    return r;
}
static inline jet j_addc(jet a, double c) { a.v += c; return a; }
static inline jet j_csub(double c, jet a) { /* c - a */
    jet r; r.v = c - a.v;
    for (int i = 0; i < NV; ++i) r.g[i] = -a.g[i];
    for (int k = 0; k < NH; ++k) r.h[k] = -a.h[k];
    return r;
}
static inline jet j_neg(jet a) { return j_csub(0.0, a); }
static inline jet j_scale(jet a, double c) {
    jet r; r.v = a.v * c;
    for (int i = 0; i < NV; ++i) r.g[i] = a.g[i] * c;
    for (int k = 0; k < NH; ++k) r.h[k] = a.h[k] * c;
    return r;
}
static inline jet j_mul(jet a, jet b) {
    jet r; r.v = a.v * b.v;
    for (int i = 0; i < NV; ++i) r.g[i] = a.v * b.g[i] + b.v * a.g[i];
    for (int k = 0; k < NH; ++k)
        r.h[k] = a.v * b.h[k] + b.v * a.h[k] + a.g[HI[k]] * b.g[HJ[k]] + a.g[HJ[k]] * b.g[HI[k]];
    return r;
}
/* f(a) given f, f', f'' at a.v */
static inline jet j_fn(jet a, double f0, double f1, double f2) {
    jet r; r.v = f0;
    for (int i = 0; i < NV; ++i) r.g[i] = f1 * a.g[i];
    for (int k = 0; k < NH; ++k) r.h[k] = f1 * a.h[k] + f2 * a.g[HI[k]] * a.g[HJ[k]];
    return r;
}
static inline jet j_exp(jet a) { double e = exp(a.v); return j_fn(a, e, e, e); }
static inline jet j_log(jet a) { double i = 1.0 / a.v; return j_fn(a, log(a.v), i, -i * i); }
static inline jet j_sqrt(jet a) {
    double s = sqrt(a.v);
    double d1 = 1.0 / (2.0 * s);
    return j_fn(a, s, d1, -d1 / (2.0 * a.v));
}
static inline jet j_inv(jet a) { double i = 1.0 / a.v; return j_fn(a, i, -i * i, 2.0 * i * i * i); }
static inline jet j_div(jet a, jet b) { return j_mul(a, j_inv(b)); }
/* ForwardDiff's abs: signbit(value) ? -x : x */
static inline jet j_abs(jet a) { return signbit(a.v) ? j_neg(a) : a; }
/* max(x, c) with a constant: the constant (zero partials) wins when x < c */
static inline jet j_maxc(jet a, double c) { return (a.v < c) ? j_const(c) : a; }

/* ------------------------------------------------------------------------- */
/* First-order jet in (mu_u, mu_d, mu_s, T) for the thermo pass              */
/* ------------------------------------------------------------------------- */
#define ND 4
typedef struct { double v, d[ND]; } dual;
static inline dual d_const(double c) { dual r; memset(&r, 0, sizeof r); r.v = c; return r; }
static inline dual d_var(double c, int i) { dual r = d_const(c); r.d[i] = 1.0; return r; }
static inline dual d_add(dual a, dual b) { dual r; r.v = a.v + b.v; for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] + b.d[i]; return r; }
static inline dual d_sub(dual a, dual b) { dual r; r.v = a.v - b.v; for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] - b.d[i]; return r; }
static inline dual d_addc(dual a, double c) { a.v += c; return a; }
static inline dual d_neg(dual a) { dual r; r.v = -a.v; for (int i = 0; i < ND; ++i) r.d[i] = -a.d[i]; return r; }
static inline dual d_scale(dual a, double c) { dual r; r.v = a.v * c; for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] * c; return r; }
static inline dual d_mul(dual a, dual b) { dual r; r.v = a.v * b.v; for (int i = 0; i < ND; ++i) r.d[i] = a.v * b.d[i] + b.v * a.d[i]; return r; }
static inline dual d_fn(dual a, double f0, double f1) { dual r; r.v = f0; for (int i = 0; i < ND; ++i) r.d[i] = f1 * a.d[i]; return r; }
static inline dual d_exp(dual a) { double e = exp(a.v); return d_fn(a, e, e); }
static inline dual d_log(dual a) { return d_fn(a, log(a.v), 1.0 / a.v); }
static inline dual d_inv(dual a) { double i = 1.0 / a.v; return d_fn(a, i, -i * i); }
static inline dual d_maxc(dual a, double c) { return (a.v < c) ? d_const(c) : a; }

/* ------------------------------------------------------------------------- */
/* Model pieces                                                              */
/* ------------------------------------------------------------------------- */
#define POLYAKOV_EPS 1e-16

typedef struct {
    int n;                  /* p_num * t_num */
    const double *p, *c, *w; /* column-major meshes, Integrals.jl:87-97 */
} or_nodes;

/* Thermodynamics.jl:81-90: M_i = m_i0 - 4 G phi_i + 2 K phi_j phi_k */
static void mass_jet(const or_params *P, const jet *x, jet *M) {
    jet four_g_u = j_scale(x[0], 4.0 * P->G), four_g_d = j_scale(x[1], 4.0 * P->G), four_g_s = j_scale(x[2], 4.0 * P->G);
    M[0] = j_add(j_csub(P->m_ud0, four_g_u), j_mul(j_scale(x[1], 2.0 * P->K), x[2]));
    M[1] = j_add(j_csub(P->m_ud0, four_g_d), j_mul(j_scale(x[0], 2.0 * P->K), x[2]));
    M[2] = j_add(j_csub(P->m_s0, four_g_s), j_mul(j_scale(x[0], 2.0 * P->K), x[1]));
}
void or_mass(const or_params *P, const double *x, double *M) {
    M[0] = P->m_ud0 - 4.0 * P->G * x[0] + 2.0 * P->K * x[1] * x[2];
    M[1] = P->m_ud0 - 4.0 * P->G * x[1] + 2.0 * P->K * x[0] * x[2];
    M[2] = P->m_s0 - 4.0 * P->G * x[2] + 2.0 * P->K * x[0] * x[1];
}

/* Integrals.jl:123-132 vacuum_integral on a jet */
static jet vacuum_jet(const or_params *P, jet m) {
    const double L = P->Lambda;
    jet ms = j_addc(j_abs(m), 1e-12);
    jet ms2 = j_mul(ms, ms);
    jet sq = j_sqrt(j_addc(ms2, L * L));
    jet poly = j_mul(j_scale(sq, L), j_addc(ms2, 2.0 * L * L));
    jet ms4 = j_mul(ms2, ms2);
    jet lt = j_mul(ms4, j_log(j_div(j_addc(sq, L), ms)));
    return j_scale(j_sub(poly, lt), 1.0 / (16.0 * M_PI * M_PI));
}
static double vacuum_plain(const or_params *P, double m) {
    const double L = P->Lambda;
    double ms = fabs(m) + 1e-12;
    double sq = sqrt(L * L + ms * ms);
    double poly = L * sq * (2.0 * L * L + ms * ms);
    double lt = ms * ms * ms * ms * log((L + sq) / ms);
    return (poly - lt) / (16.0 * M_PI * M_PI);
}
double or_vacuum_integral(const or_params *P, double m) { return vacuum_plain(P, m); }

/* Integrals.jl:193-238 calculate_log_term: ln f+ + ln f- with the log-sum-exp branches */
static jet log_term_jet(jet E, double mu, double T, jet Phi, jet Phib) {
    const double invT = 1.0 / T;
    jet a = j_scale(j_addc(E, -mu), -invT);
    jet b = j_scale(j_addc(E, mu), -invT);
    jet lfp, lfm;
    jet threePhi = j_scale(Phi, 3.0), threePhib = j_scale(Phib, 3.0);
    if (a.v > 0) {
        jet m_a = j_scale(a, 3.0);
        jet e1 = j_exp(j_scale(a, -2.0));
        jet e2 = j_exp(j_neg(a));
        jet e0 = j_exp(j_neg(m_a));
        jet term = j_addc(j_add(j_add(e0, j_mul(threePhi, e1)), j_mul(threePhib, e2)), 1.0);
        lfp = j_add(m_a, j_log(j_maxc(term, POLYAKOV_EPS)));
    } else {
        jet e1 = j_exp(a);
        jet e2 = j_mul(e1, e1);
        jet e3 = j_mul(e1, e2);
        jet f = j_add(j_add(j_addc(j_mul(threePhi, e1), 1.0), j_mul(threePhib, e2)), e3);
        lfp = j_log(j_maxc(f, POLYAKOV_EPS));
    }
    if (b.v > 0) {
        jet m_b = j_scale(b, 3.0);
        jet e1 = j_exp(j_scale(b, -2.0));
        jet e2 = j_exp(j_neg(b));
        jet e0 = j_exp(j_neg(m_b));
        jet term = j_addc(j_add(j_add(e0, j_mul(threePhib, e1)), j_mul(threePhi, e2)), 1.0);
        lfm = j_add(m_b, j_log(j_maxc(term, POLYAKOV_EPS)));
    } else {
        jet e1 = j_exp(b);
        jet e2 = j_mul(e1, e1);
        jet e3 = j_mul(e1, e2);
        jet f = j_add(j_add(j_addc(j_mul(threePhib, e1), 1.0), j_mul(threePhi, e2)), e3);
        lfm = j_log(j_maxc(f, POLYAKOV_EPS));
    }
    return j_add(lfp, lfm);
}

/* Thermodynamics.jl:124-130 calculate_U with safe_log (Integrals.jl:159-162) */
static jet U_jet(const or_params *P, double T, jet Phi, jet Phib) {
    const double r = P->T0 / T;
    const double Ta = P->a0 + P->a1 * r + P->a2 * r * r;
    const double Tb = P->b3 * r * r * r;
    jet pp = j_mul(Phib, Phi);
    jet cub = j_add(j_mul(j_mul(Phib, Phib), Phib), j_mul(j_mul(Phi, Phi), Phi));
    jet val = j_sub(j_add(j_csub(1.0, j_scale(pp, 6.0)), j_scale(cub, 4.0)), j_scale(j_mul(pp, pp), 3.0));
    jet lg;
    if (val.v <= 0 || val.v < POLYAKOV_EPS) lg = j_const(log(POLYAKOV_EPS));
    else lg = j_log(val);
    const double T4 = T * T * T * T;
    return j_scale(j_add(j_scale(pp, -0.5 * Ta), j_scale(lg, Tb)), T4);
}

/* Thermodynamics.jl:181-195 calculate_omega on jets in x (T, mu, xi plain) */
static jet omega_jet(const or_params *P, const or_nodes *nd, const double *xv, const double *mu, double T, double xi) {
    jet x[NV];
    for (int i = 0; i < NV; ++i) x[i] = j_var(xv[i], i);
    /* chi: Thermodynamics.jl:112-114 */
    jet sq = j_add(j_add(j_mul(x[0], x[0]), j_mul(x[1], x[1])), j_mul(x[2], x[2]));
    jet pr = j_mul(j_mul(x[0], x[1]), x[2]);
    jet chi = j_sub(j_scale(sq, 2.0 * P->G), j_scale(pr, 4.0 * P->K));
    jet U = U_jet(P, T, x[3], x[4]);
    jet M[3];
    mass_jet(P, x, M);
    /* Integrals.jl:139-145 */
    jet vac = j_add(j_add(vacuum_jet(P, M[0]), vacuum_jet(P, M[1])), vacuum_jet(P, M[2]));
    jet esum = j_scale(vac, -2.0 * P->N_color);
    /* Integrals.jl:248-259 */
    jet total = j_const(0.0);
    for (int f = 0; f < 3; ++f) {
        jet M2 = j_mul(M[f], M[f]);
        for (int k = 0; k < nd->n; ++k) {
            const double p = nd->p[k], c = nd->c[k];
            const double pc = p * c;
            jet E = j_sqrt(j_addc(j_addc(M2, p * p), xi * (pc * pc)));
            jet L = log_term_jet(E, mu[f], T, x[3], x[4]);
            total = j_add(total, j_scale(L, nd->w[k]));
        }
    }
    jet logsum = j_scale(total, -2.0 * T);
    return j_add(j_add(j_add(chi, U), esum), logsum);
}

/* ---- thermo pass on first-order duals in (mu_u, mu_d, mu_s, T) ---- */
static dual log_term_dual(double E, dual mu, dual T, double Phi, double Phib) {
    dual invT = d_inv(T);
    dual a = d_mul(d_neg(d_addc(d_neg(mu), E)), invT);  /* -(E - mu)/T */
    dual b = d_mul(d_neg(d_add(mu, d_const(E))), invT);  /* -(E + mu)/T */
    dual lfp, lfm;
    if (a.v > 0) {
        dual m_a = d_scale(a, 3.0);
        dual e1 = d_exp(d_scale(a, -2.0)), e2 = d_exp(d_neg(a)), e0 = d_exp(d_neg(m_a));
        dual term = d_addc(d_add(d_add(e0, d_scale(e1, 3.0 * Phi)), d_scale(e2, 3.0 * Phib)), 1.0);
        lfp = d_add(m_a, d_log(d_maxc(term, POLYAKOV_EPS)));
    } else {
        dual e1 = d_exp(a), e2 = d_mul(e1, e1), e3 = d_mul(e1, e2);
        dual f = d_add(d_add(d_addc(d_scale(e1, 3.0 * Phi), 1.0), d_scale(e2, 3.0 * Phib)), e3);
        lfp = d_log(d_maxc(f, POLYAKOV_EPS));
    }
    if (b.v > 0) {
        dual m_b = d_scale(b, 3.0);
        dual e1 = d_exp(d_scale(b, -2.0)), e2 = d_exp(d_neg(b)), e0 = d_exp(d_neg(m_b));
        dual term = d_addc(d_add(d_add(e0, d_scale(e1, 3.0 * Phib)), d_scale(e2, 3.0 * Phi)), 1.0);
        lfm = d_add(m_b, d_log(d_maxc(term, POLYAKOV_EPS)));
    } else {
        dual e1 = d_exp(b), e2 = d_mul(e1, e1), e3 = d_mul(e1, e2);
        dual f = d_add(d_add(d_addc(d_scale(e1, 3.0 * Phib), 1.0), d_scale(e2, 3.0 * Phi)), e3);
        lfm = d_log(d_maxc(f, POLYAKOV_EPS));
    }
    return d_add(lfp, lfm);
}

static dual U_dual(const or_params *P, dual T, double Phi, double Phib) {
    dual r = d_scale(d_inv(T), P->T0);
    dual Ta = d_addc(d_add(d_scale(r, P->a1), d_scale(d_mul(r, r), P->a2)), P->a0);
    dual Tb = d_scale(d_mul(d_mul(r, r), r), P->b3);
    double val = 1.0 - 6.0 * Phib * Phi + 4.0 * (Phib * Phib * Phib + Phi * Phi * Phi) - 3.0 * (Phib * Phi) * (Phib * Phi);
    double lg = (val <= 0 || val < POLYAKOV_EPS) ? log(POLYAKOV_EPS) : log(val);
    dual T2 = d_mul(T, T);
    dual T4 = d_mul(T2, T2);
    return d_mul(T4, d_add(d_scale(Ta, -0.5 * Phib * Phi), d_scale(Tb, lg)));
}

/* Omega with (mu, T) as duals and x plain: value = Omega, d[0..2] = dOmega/dmu_f, d[3] = dOmega/dT */
static dual omega_dual(const or_params *P, const or_nodes *nd, const double *x, const double *mu, double T, double xi) {
    dual muv[3] = {d_var(mu[0], 0), d_var(mu[1], 1), d_var(mu[2], 2)};
    dual Td = d_var(T, 3);
    double chi = 2.0 * P->G * (x[0] * x[0] + x[1] * x[1] + x[2] * x[2]) - 4.0 * P->K * (x[0] * x[1] * x[2]);
    dual U = U_dual(P, Td, x[3], x[4]);
    double M[3];
    or_mass(P, x, M);
    double esum = -2.0 * P->N_color * (vacuum_plain(P, M[0]) + vacuum_plain(P, M[1]) + vacuum_plain(P, M[2]));
    dual total = d_const(0.0);
    for (int f = 0; f < 3; ++f) {
        for (int k = 0; k < nd->n; ++k) {
            const double p = nd->p[k], c = nd->c[k], pc = p * c;
            double E = sqrt(p * p + M[f] * M[f] + xi * (pc * pc));
            dual L = log_term_dual(E, muv[f], Td, x[3], x[4]);
            total = d_add(total, d_scale(L, nd->w[k]));
        }
    }
    dual logsum = d_mul(d_scale(Td, -2.0), total);
    return d_add(d_addc(U, chi + esum), logsum);
}

/* QuarkDistribution.jl:14-51 (with the exp clamp to [1e-200, 1e200]) */
static double quark_dist(double E, double mu, double T, double Phi, double Phib) {
    double beta = 1.0 / T;
    double e = exp(-(E - mu) * beta);
    if (e < 1e-200) e = 1e-200;
    if (e > 1e200) e = 1e200;
    double e2 = e * e, e3 = e2 * e;
    return (Phi * e + 2.0 * Phib * e2 + e3) / (1.0 + 3.0 * Phi * e + 3.0 * Phib * e2 + e3);
}
static double antiquark_dist(double E, double mu, double T, double Phi, double Phib) {
    double beta = 1.0 / T;
    double e = exp(-(E + mu) * beta);
    if (e < 1e-200) e = 1e-200;
    if (e > 1e200) e = 1e200;
    double e2 = e * e, e3 = e2 * e;
    return (Phib * e + 2.0 * Phi * e2 + e3) / (1.0 + 3.0 * Phib * e + 3.0 * Phi * e2 + e3);
}

/* ------------------------------------------------------------------------- */
/* Public evaluation API                                                     */
/* ------------------------------------------------------------------------- */
/* Omega, grad_x Omega, Hessian_x Omega (row-major 5x5) */
void or_eval(const or_params *P, int n_nodes, const double *pm, const double *cm, const double *wm,
             const double *x, const double *mu, double T, double xi,
             double *omega, double *grad, double *hess) {
    or_nodes nd = {n_nodes, pm, cm, wm};
    jet o = omega_jet(P, &nd, x, mu, T, xi);
    *omega = o.v;
    for (int i = 0; i < NV; ++i) grad[i] = o.g[i];
    for (int k = 0; k < NH; ++k) {
        hess[HI[k] * NV + HJ[k]] = o.h[k];
        hess[HJ[k] * NV + HI[k]] = o.h[k];
    }
}

/* calculate_thermo (Thermodynamics.jl:233-244) + calculate_number_densities (:255-281).
 * out: pressure, rho_norm, entropy, energy, rho[3], nq[3], naq[3] */
typedef struct {
    double pressure, rho_norm, entropy, energy;
    double rho[3], nq[3], naq[3];
} or_thermo;

void or_thermo_eval(const or_params *P, int n_nodes, const double *pm, const double *cm, const double *wm,
                    const double *x, const double *mu, double T, double xi, or_thermo *th) {
    or_nodes nd = {n_nodes, pm, cm, wm};
    dual o = omega_dual(P, &nd, x, mu, T, xi);
    double pressure = -o.v;
    double rho[3] = {-o.d[0], -o.d[1], -o.d[2]};
    double entropy = -o.d[3];
    th->pressure = pressure;
    th->rho_norm = (rho[0] + rho[1] + rho[2]) / (3.0 * P->rho0);
    th->entropy = entropy;
    th->energy = -pressure + (mu[0] * rho[0] + mu[1] * rho[1] + mu[2] * rho[2]) + T * entropy;
    for (int i = 0; i < 3; ++i) th->rho[i] = rho[i];
    double M[3];
    or_mass(P, x, M);
    const double pref = 2.0 * P->N_color;
    for (int f = 0; f < 3; ++f) {
        double tq = 0.0, ta = 0.0;
        for (int k = 0; k < n_nodes; ++k) {
            const double p = pm[k], c = cm[k], w = wm[k];
            double E = sqrt(p * p + M[f] * M[f] + xi * (p * c) * (p * c));
            tq += w * pref * quark_dist(E, mu[f], T, x[3], x[4]);
            ta += w * pref * antiquark_dist(E, mu[f], T, x[3], x[4]);
        }
        th->nq[f] = tq;
        th->naq[f] = ta;
    }
}

/* ------------------------------------------------------------------------- */
/* Dense 5x5 linear algebra                                                  */
/* ------------------------------------------------------------------------- */
/* LU with partial pivoting (first maximal |a| in the column, as LAPACK getrf picks);
 * returns 0 on success, 1 when a pivot is exactly zero (Julia raises SingularException). */
static int lu_solve(int n, const double *Ain, const double *b, double *x) {
    double A[25], y[5];
    memcpy(A, Ain, sizeof(double) * n * n);
    memcpy(y, b, sizeof(double) * n);
    int piv[5];
    for (int k = 0; k < n; ++k) {
        int p = k;
        double best = fabs(A[k * n + k]);
        for (int i = k + 1; i < n; ++i)
            if (fabs(A[i * n + k]) > best) { best = fabs(A[i * n + k]); p = i; }
        piv[k] = p;
        if (A[p * n + k] == 0.0) return 1;
        if (p != k)
            for (int j = 0; j < n; ++j) { double t = A[k * n + j]; A[k * n + j] = A[p * n + j]; A[p * n + j] = t; }
        for (int i = k + 1; i < n; ++i) {
            double l = A[i * n + k] / A[k * n + k];
            A[i * n + k] = l;
            for (int j = k + 1; j < n; ++j) A[i * n + j] -= l * A[k * n + j];
        }
    }
    for (int k = 0; k < n; ++k) {
        int p = piv[k];
        if (p != k) { double t = y[k]; y[k] = y[p]; y[p] = t; }
    }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < i; ++j) y[i] -= A[i * n + j] * y[j];
    for (int i = n - 1; i >= 0; --i) {
        for (int j = i + 1; j < n; ++j) y[i] -= A[i * n + j] * y[j];
        y[i] /= A[i * n + i];
    }
    memcpy(x, y, sizeof(double) * n);
    return 0;
}

static double norm_inf(const double *v, int n) {
    double m = 0.0;
    for (int i = 0; i < n; ++i) {
        double a = fabs(v[i]);
        if (isnan(a)) return NAN;
        if (a > m) m = a;
    }
    return m;
}
static int any_nan(const double *v, int n) { for (int i = 0; i < n; ++i) if (isnan(v[i])) return 1; return 0; }
static int all_finite(const double *v, int n) { for (int i = 0; i < n; ++i) if (!isfinite(v[i])) return 0; return 1; }

/* ------------------------------------------------------------------------- */
/* Residual F = grad_x P and Jacobian J = Hessian_x P  (Conditions.jl:72-86)  */
/* ------------------------------------------------------------------------- */
typedef struct {
    const or_params *P;
    or_nodes nd;
    double mu[3], T, xi;
    long evals; /* residual+Jacobian evaluations (each is one pass over 3*p*t nodes) */
} or_problem;

static void residual_jacobian(or_problem *pb, const double *x, double *F, double *J) {
    jet o = omega_jet(pb->P, &pb->nd, x, pb->mu, pb->T, pb->xi);
    pb->evals++;
    for (int i = 0; i < NV; ++i) F[i] = -o.g[i];
    for (int k = 0; k < NH; ++k) {
        J[HI[k] * NV + HJ[k]] = -o.h[k];
        J[HJ[k] * NV + HI[k]] = -o.h[k];
    }
}

typedef struct {
    double x[5];
    double residual_norm;
    int iterations;
    int f_converged, x_converged;
    int exception; /* NLsolve raised (non-finite initial residual) */
} or_nl_result;

/* NLsolve :newton with the static line search (full step), restated:
 *   F0,J0 at x0; non-finite F0 raises; converged iff ||F||_inf < ftol or
 *   ||x - x_prev||_inf < xtol; singular J -> Levenberg-Marquardt direction
 *   -(J'J + lambda I) \ J'F with lambda = 1e6 sqrt(n eps) sum|J'J|. */
static void newton_solve(or_problem *pb, const double *x0, int max_iter, double xtol, double ftol, or_nl_result *r) {
    double x[5], xold[5], F[5], J[25], p[5];
    memcpy(x, x0, sizeof x);
    for (int i = 0; i < 5; ++i) xold[i] = NAN;
    memset(r, 0, sizeof *r);
    residual_jacobian(pb, x, F, J);
    if (!all_finite(F, 5)) { r->exception = 1; memcpy(r->x, x, sizeof x); r->residual_norm = NAN; return; }
    int it = 0;
    int xconv = 0, fconv = norm_inf(F, 5) < ftol;
    int stopped = any_nan(x, 5) || any_nan(F, 5);
    int converged = xconv || fconv;
    while (!stopped && !converged && it < max_iter) {
        ++it;
        if (lu_solve(5, J, F, p) != 0) {
            double g[5], JJ[25], s = 0.0;
            for (int i = 0; i < 5; ++i) { g[i] = 0.0; for (int k = 0; k < 5; ++k) g[i] += J[k * 5 + i] * F[k]; }
            for (int i = 0; i < 5; ++i)
                for (int j = 0; j < 5; ++j) {
                    double a = 0.0;
                    for (int k = 0; k < 5; ++k) a += J[k * 5 + i] * J[k * 5 + j];
                    JJ[i * 5 + j] = a;
                    s += fabs(a);
                }
            double lambda = 1e6 * sqrt(5.0 * 2.220446049250313e-16) * s;
            double A[25];
            for (int i = 0; i < 25; ++i) A[i] = -JJ[i];
            for (int i = 0; i < 5; ++i) A[i * 5 + i] -= lambda;
            if (lu_solve(5, A, g, p) != 0) for (int i = 0; i < 5; ++i) p[i] = NAN;
        } else {
            for (int i = 0; i < 5; ++i) p[i] = -p[i];
        }
        memcpy(xold, x, sizeof x);
        for (int i = 0; i < 5; ++i) x[i] += p[i];
        residual_jacobian(pb, x, F, J);
        double dx = 0.0;
        int dx_nan = 0;
        for (int i = 0; i < 5; ++i) { double d = fabs(x[i] - xold[i]); if (isnan(d)) dx_nan = 1; if (d > dx) dx = d; }
        xconv = !any_nan(xold, 5) && !dx_nan && dx < xtol;
        fconv = norm_inf(F, 5) < ftol;
        stopped = any_nan(x, 5) || any_nan(F, 5);
        converged = xconv || fconv;
    }
    memcpy(r->x, x, sizeof x);
    r->residual_norm = norm_inf(F, 5);
    r->iterations = it;
    r->f_converged = fconv;
    r->x_converged = xconv;
}

static double wnorm(const double *d, const double *v) {
    double s = 0.0;
    for (int i = 0; i < 5; ++i) s += (d[i] * v[i]) * (d[i] * v[i]);
    return sqrt(s);
}

/* Powell dogleg step inside the scaled trust region ||D p|| <= delta (Nocedal & Wright 4.1) */
static void dogleg(double *p, const double *r, const double *d, const double *J, double delta) {
    double pi[5], pc[5], g[5];
    if (lu_solve(5, J, r, pi) != 0) {
        /* singular: minimum-norm least squares via normal equations with a tiny ridge */
        double JJ[25], Jr[5];
        for (int i = 0; i < 5; ++i) { Jr[i] = 0.0; for (int k = 0; k < 5; ++k) Jr[i] += J[k * 5 + i] * r[k]; }
        for (int i = 0; i < 5; ++i)
            for (int j = 0; j < 5; ++j) { double a = 0.0; for (int k = 0; k < 5; ++k) a += J[k * 5 + i] * J[k * 5 + j]; JJ[i * 5 + j] = a; }
        for (int i = 0; i < 5; ++i) JJ[i * 5 + i] += 2.220446049250313e-16 * (1.0 + JJ[i * 5 + i]);
        if (lu_solve(5, JJ, Jr, pi) != 0) for (int i = 0; i < 5; ++i) pi[i] = 0.0;
    }
    for (int i = 0; i < 5; ++i) pi[i] = -pi[i];
    if (wnorm(d, pi) <= delta) { memcpy(p, pi, sizeof pi); return; }
    for (int i = 0; i < 5; ++i) { double a = 0.0; for (int k = 0; k < 5; ++k) a += J[k * 5 + i] * r[k]; g[i] = a / (d[i] * d[i]); }
    double Jg2 = 0.0;
    for (int k = 0; k < 5; ++k) { double a = 0.0; for (int i = 0; i < 5; ++i) a += J[k * 5 + i] * g[i]; Jg2 += a * a; }
    double wg = wnorm(d, g);
    for (int i = 0; i < 5; ++i) pc[i] = -(wg * wg) / Jg2 * g[i];
    if (wnorm(d, pc) >= delta) {
        for (int i = 0; i < 5; ++i) p[i] = g[i] * (-delta / wg);
        return;
    }
    double pd[5];
    for (int i = 0; i < 5; ++i) pd[i] = pi[i] - pc[i];
    double bq = 0.0;
    for (int i = 0; i < 5; ++i) bq += (d[i] * pc[i]) * (d[i] * pd[i]);
    bq *= 2.0;
    double aq = wnorm(d, pd);
    aq *= aq;
    double wpc = wnorm(d, pc);
    double tau = (-bq + sqrt(bq * bq - 4.0 * aq * (wpc * wpc - delta * delta))) / (2.0 * aq);
    for (int i = 0; i < 5; ++i) p[i] = pc[i] + tau * pd[i];
}

/* NLsolve :trust_region (dogleg, autoscale=true, factor=1), restated */
static void trust_region_solve(or_problem *pb, const double *x0, int max_iter, double xtol, double ftol, or_nl_result *res) {
    double x[5], xold[5], r[5], F[5], J[25], Jacc[25], d[5], p[5], rp[5];
    memcpy(x, x0, sizeof x);
    for (int i = 0; i < 5; ++i) xold[i] = NAN;
    memset(res, 0, sizeof *res);
    residual_jacobian(pb, x, F, J);
    memcpy(r, F, sizeof r);
    memcpy(Jacc, J, sizeof J);
    if (!all_finite(r, 5)) { res->exception = 1; memcpy(res->x, x, sizeof x); res->residual_norm = NAN; return; }
    int it = 0;
    int xconv = 0, fconv = norm_inf(r, 5) < ftol;
    int stopped = any_nan(x, 5) || any_nan(F, 5);
    int converged = xconv || fconv;
    if (!converged) {
        for (int j = 0; j < 5; ++j) {
            double s = 0.0;
            for (int i = 0; i < 5; ++i) s += Jacc[i * 5 + j] * Jacc[i * 5 + j];
            d[j] = sqrt(s);
            if (d[j] == 0.0) d[j] = 1.0;
        }
        double delta = wnorm(d, x);
        if (delta == 0.0) delta = 1.0;
        const double eta = 1e-4;
        while (!stopped && !converged && it < max_iter) {
            ++it;
            dogleg(p, r, d, Jacc, delta);
            memcpy(xold, x, sizeof x);
            for (int i = 0; i < 5; ++i) x[i] += p[i];
            residual_jacobian(pb, x, F, J);
            for (int k = 0; k < 5; ++k) { double a = 0.0; for (int i = 0; i < 5; ++i) a += Jacc[k * 5 + i] * p[i]; rp[k] = a + r[k]; }
            double sr = 0.0, sf = 0.0, sp = 0.0;
            for (int i = 0; i < 5; ++i) { sr += r[i] * r[i]; sf += F[i] * F[i]; sp += rp[i] * rp[i]; }
            double rho = (sr - sf) / (sr - sp);
            if (rho > eta) {
                memcpy(r, F, sizeof r);
                memcpy(Jacc, J, sizeof J);
                for (int j = 0; j < 5; ++j) {
                    double s = 0.0;
                    for (int i = 0; i < 5; ++i) s += Jacc[i * 5 + j] * Jacc[i * 5 + j];
                    double cn = sqrt(s);
                    d[j] = (0.1 * d[j] > cn) ? 0.1 * d[j] : cn;
                }
                double dx = 0.0;
                int dxn = 0;
                for (int i = 0; i < 5; ++i) { double dd = fabs(x[i] - xold[i]); if (isnan(dd)) dxn = 1; if (dd > dx) dx = dd; }
                xconv = !dxn && dx < xtol;
                fconv = norm_inf(r, 5) < ftol;
                converged = xconv || fconv;
            } else {
                for (int i = 0; i < 5; ++i) x[i] -= p[i];
                xconv = 0;
                converged = 0;
            }
            if (rho < 0.1) delta = delta / 2.0;
            else if (rho >= 0.9) delta = 2.0 * wnorm(d, p);
            else if (rho >= 0.5) { double t = 2.0 * wnorm(d, p); if (t > delta) delta = t; }
            stopped = any_nan(x, 5) || any_nan(F, 5);
        }
    }
    memcpy(res->x, x, sizeof x);
    res->residual_norm = norm_inf(r, 5);
    res->iterations = it;
    res->f_converged = fconv;
    res->x_converged = xconv;
}

/* ------------------------------------------------------------------------- */
/* SolverResult and the solve() paths                                        */
/* ------------------------------------------------------------------------- */
typedef struct {
    int converged;
    double x[5];
    double omega, pressure, rho_norm, entropy, energy;
    double masses[3];
    int iterations;
    double residual_norm;
    double rho[3], nq[3], naq[3];
    int f_converged, phys;
    int status;       /* 0 ok (converged), 1 not converged, 2 exception (seed skipped), 3 all seeds failed */
    int chosen_seed;  /* index in the seed list (-1: single-seed primary) */
    int used_fallback;/* 1 when the trust-region candidate was chosen */
    long evals;       /* residual+Jacobian passes spent on this point */
} or_result;

typedef struct {
    int max_iter;            /* NLsolve iterations (reference default 1000; scan script 40) */
    double ftol, xtol;       /* reference: 1e-9, 1e-9 */
    double residual_norm_max;/* 1e-6 */
    double phi_tol;          /* 1e-8 */
    double omega_tie_rtol;   /* Omega within rtol*|Omega| of the kept candidate counts as a tie */
    int trust_region_fallback;
    int auto_multiseed_fallback;
} or_opts;

void or_opts_default(or_opts *o) {
    o->max_iter = 1000;
    o->ftol = 1e-9;
    o->xtol = 1e-9;
    o->residual_norm_max = 1e-6;
    o->phi_tol = 1e-8;
    o->omega_tie_rtol = 1e-12;
    o->trust_region_fallback = 1;
    o->auto_multiseed_fallback = 1;
}

typedef struct {
    int phys;
    double x[5];
    double omega, pressure, rho_norm, entropy, energy, masses[3];
    double rho[3], nq[3], naq[3];
} candidate;

/* ImplicitSolver.jl:50-70 postprocess + physicality */
static void postprocess(or_problem *pb, const or_opts *o, const double *x, candidate *c) {
    or_thermo th;
    or_thermo_eval(pb->P, pb->nd.n, pb->nd.p, pb->nd.c, pb->nd.w, x, pb->mu, pb->T, pb->xi, &th);
    memcpy(c->x, x, sizeof(double) * 5);
    c->pressure = th.pressure;
    c->omega = -th.pressure;
    c->rho_norm = th.rho_norm;
    c->entropy = th.entropy;
    c->energy = th.energy;
    or_mass(pb->P, x, c->masses);
    memcpy(c->rho, th.rho, sizeof th.rho);
    memcpy(c->nq, th.nq, sizeof th.nq);
    memcpy(c->naq, th.naq, sizeof th.naq);
    const double Phi = x[3], Phib = x[4], tol = o->phi_tol;
    int ok = isfinite(Phi) && isfinite(Phib) && (-tol <= Phi && Phi <= 1 + tol) && (-tol <= Phib && Phib <= 1 + tol);
    if (ok) for (int i = 0; i < 3; ++i) if (!isfinite(c->masses[i]) || c->masses[i] <= 0.0) ok = 0;
    if (ok) ok = isfinite(c->omega) && isfinite(c->pressure) && isfinite(c->rho_norm) && isfinite(c->entropy) && isfinite(c->energy);
    c->phys = ok;
}

static int good(const or_nl_result *r, const candidate *c, double rmax) {
    return r->f_converged && isfinite(r->residual_norm) && r->residual_norm <= rmax && c->phys;
}

/* ImplicitSolver.jl:72-101 _choose_candidate: returns 1 for the fallback */
static int choose_fallback(const or_nl_result *pr, const candidate *pc, const or_nl_result *fr, const candidate *fc, double rmax) {
    int pg = good(pr, pc, rmax), fg = good(fr, fc, rmax);
    if (fg && !pg) return 1;
    if (pg && !fg) return 0;
    if (fg && pg) {
        if (fc->omega < pc->omega) return 1;
        if (fc->omega > pc->omega) return 0;
        return fr->residual_norm < pr->residual_norm;
    }
    if (fr->f_converged && !pr->f_converged) return 1;
    if (pr->f_converged && !fr->f_converged) return 0;
    if (isfinite(fr->residual_norm) && isfinite(pr->residual_norm)) return fr->residual_norm < pr->residual_norm;
    return 0;
}

static void fill_result(or_result *out, const or_nl_result *r, const candidate *c, double rmax) {
    out->converged = r->f_converged && c->phys && isfinite(r->residual_norm) && r->residual_norm <= rmax;
    memcpy(out->x, c->x, sizeof c->x);
    out->omega = c->omega; out->pressure = c->pressure; out->rho_norm = c->rho_norm;
    out->entropy = c->entropy; out->energy = c->energy;
    memcpy(out->masses, c->masses, sizeof c->masses);
    memcpy(out->rho, c->rho, sizeof c->rho);
    memcpy(out->nq, c->nq, sizeof c->nq);
    memcpy(out->naq, c->naq, sizeof c->naq);
    out->iterations = r->iterations;
    out->residual_norm = r->residual_norm;
    out->f_converged = r->f_converged;
    out->phys = c->phys;
    out->status = out->converged ? 0 : 1;
}

/* solve(FixedMu) single-seed path (ImplicitSolver.jl:261-304) without the MultiSeed fallback.
 * Returns 0, or 2 when NLsolve raised (the reference propagates the exception). */
static int solve_one_seed(or_problem *pb, const double *x0, const or_opts *o, or_result *out) {
    or_nl_result pr, fr;
    candidate pc, fc;
    newton_solve(pb, x0, o->max_iter, o->xtol, o->ftol, &pr);
    if (pr.exception) { memset(out, 0, sizeof *out); out->status = 2; for (int i = 0; i < 5; ++i) out->x[i] = x0[i]; out->residual_norm = NAN; return 2; }
    postprocess(pb, o, pr.x, &pc);
    int need = o->trust_region_fallback &&
               (!pr.f_converged || !isfinite(pr.residual_norm) || pr.residual_norm > o->residual_norm_max || !pc.phys);
    out->used_fallback = 0;
    if (!need) { fill_result(out, &pr, &pc, o->residual_norm_max); return 0; }
    trust_region_solve(pb, x0, o->max_iter, o->xtol, o->ftol, &fr);
    if (fr.exception) { fill_result(out, &pr, &pc, o->residual_norm_max); return 0; }
    postprocess(pb, o, fr.x, &fc);
    if (choose_fallback(&pr, &pc, &fr, &fc, o->residual_norm_max)) {
        fill_result(out, &fr, &fc, o->residual_norm_max);
        out->used_fallback = 1;
    } else {
        fill_result(out, &pr, &pc, o->residual_norm_max);
    }
    return 0;
}

/* solve_multi (ImplicitSolver.jl:532-559): every seed, keep converged ones, argmin Omega
 * (first minimum wins, SeedStrategies.jl:236-240).  Candidates are visited in seed order and a
 * later one replaces the kept one only when its Omega is lower by more than
 * omega_tie_rtol*|Omega| (several seeds that land on the same solution differ only by
 * rounding).  status 3 when none converged. */
static void solve_multi(or_problem *pb, int n_seeds, const double *seeds, const or_opts *o, or_result *out) {
    or_result best, cur, first_seen;
    int have = 0, any = 0;
    memset(&first_seen, 0, sizeof first_seen);
    for (int s = 0; s < n_seeds; ++s) {
        int rc = solve_one_seed(pb, seeds + 5 * s, o, &cur);
        if (rc == 2) continue;
        cur.chosen_seed = s;
        if (!any) { first_seen = cur; any = 1; }
        if (!cur.converged) continue;
        if (!have || cur.omega < best.omega - o->omega_tie_rtol * fabs(best.omega)) { best = cur; have = 1; }
    }
    if (have) { *out = best; out->status = 0; return; }
    if (any) { *out = first_seen; } else { memset(out, 0, sizeof *out); out->residual_norm = NAN; out->chosen_seed = -1; }
    out->converged = 0;
    out->status = 3;
}

/* The reference's built-in seeds (SeedStrategies.jl:56-95) */
static const double HADRON_SEED[5] = {-1.84329, -1.84329, -2.22701, 1.0e-5, 4.0e-5};
static const double MEDIUM_SEED[5] = {-1.3647, -1.3647, -2.14502, 0.10594, 0.15569};
static const double HIGH_DENSITY_SEED[5] = {-0.21695, -0.21695, -2.01372, 0.18601, 0.22333};
static const double HIGH_TEMP_SEED[5] = {-0.73192, -0.73192, -1.79539, 0.60532, 0.60532};
static const double VERY_HIGH_TEMP_SEED[5] = {-0.30, -0.30, -0.90, 0.90, 0.90};
static const double HT_0p8_SEED[5] = {-0.50, -0.50, -1.20, 0.80, 0.80};
static const double HT_0p9_SEED[5] = {-0.30, -0.30, -0.90, 0.90, 0.90};
static const double HT_0p95_SEED[5] = {-0.20, -0.20, -0.70, 0.95, 0.95};
static const double WEAK_CHIRAL_CONF_SEED[5] = {-0.50, -0.50, -1.20, 1e-3, 1e-3};

/* get_all_seeds(MultiSeed()) (SeedStrategies.jl:257-284); candidate 2 is DefaultSeed(:quark),
 * which becomes VERY_HIGH_TEMP at T >= 300 MeV (:204-225).  Returns the number of seeds. */
int or_multiseed_seeds(const or_params *P, double T_fm, double *out /* 6*5 */) {
    const double *list[6] = {HADRON_SEED, HIGH_TEMP_SEED, WEAK_CHIRAL_CONF_SEED, HT_0p8_SEED, HT_0p9_SEED, HT_0p95_SEED};
    if (T_fm * 197.327 >= 300.0) list[1] = VERY_HIGH_TEMP_SEED;
    (void)P;
    for (int s = 0; s < 6; ++s) memcpy(out + 5 * s, list[s], sizeof(double) * 5);
    return 6;
}

/* Named seed lookup for the host mirror: 0 hadron, 1 medium, 2 high density, 3 high temp (quark),
 * 4 very high temp, 5 HT 0.8, 6 HT 0.9, 7 HT 0.95, 8 weak chiral/confined */
int or_builtin_seed(int which, double *out) {
    const double *list[9] = {HADRON_SEED, MEDIUM_SEED, HIGH_DENSITY_SEED, HIGH_TEMP_SEED, VERY_HIGH_TEMP_SEED,
                             HT_0p8_SEED, HT_0p9_SEED, HT_0p95_SEED, WEAK_CHIRAL_CONF_SEED};
    if (which < 0 || which > 8) return -1;
    memcpy(out, list[which], sizeof(double) * 5);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Point solve entry (mode: 0 = single seed [+ auto MultiSeed fallback],      */
/*                          1 = seed list with min-Omega selection)           */
/* ------------------------------------------------------------------------- */
void or_solve_point(const or_params *P, int n_nodes, const double *pm, const double *cm, const double *wm,
                    double T, const double *mu, double xi, int mode, int n_seeds, const double *seeds,
                    const or_opts *o, or_result *out) {
    or_problem pb;
    pb.P = P; pb.nd.n = n_nodes; pb.nd.p = pm; pb.nd.c = cm; pb.nd.w = wm;
    pb.mu[0] = mu[0]; pb.mu[1] = mu[1]; pb.mu[2] = mu[2];
    pb.T = T; pb.xi = xi; pb.evals = 0;
    if (mode == 1) {
        solve_multi(&pb, n_seeds, seeds, o, out);
    } else {
        int rc = solve_one_seed(&pb, seeds, o, out);
        out->chosen_seed = -1;
        /* A non-finite initial residual raises inside nlsolve before the fallback is reached
         * (ImplicitSolver.jl:112 is outside any try), so status 2 is returned as is. */
        if (rc != 2 && !out->converged && o->auto_multiseed_fallback) {
            /* ImplicitSolver.jl:306-327: fall back to MultiSeed(); keep the single result if that throws */
            or_result single = *out, multi;
            double ms[30];
            int ns = or_multiseed_seeds(P, T, ms);
            or_opts o2 = *o;
            o2.auto_multiseed_fallback = 0;
            solve_multi(&pb, ns, ms, &o2, &multi);
            if (multi.status == 0) *out = multi;
            else *out = single;
        }
    }
    out->evals = pb.evals;
}

/* Batched driver over points (OpenMP over points; this is the CPU baseline loop).
 * Inputs SoA: T[n], mu[3n] (mu_u, mu_d, mu_s per point), xi[n]; seeds as in or_solve_point
 * (mode 0: seeds is [n x 5] per point; mode 1: a shared [n_seeds x 5] table, and when
 * multiseed_rule != 0 the table is rebuilt per point by or_multiseed_seeds). */
void or_solve_batch(const or_params *P, int n_nodes, const double *pm, const double *cm, const double *wm,
                    long n, const double *T, const double *mu, const double *xi,
                    int mode, int n_seeds, const double *seeds, int multiseed_rule,
                    const or_opts *o, or_result *out, int n_threads) {
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#else
    (void)n_threads;
#endif
#pragma omp parallel for schedule(dynamic, 1)
    for (long i = 0; i < n; ++i) {
        const double *sd = seeds;
        double tbl[30];
        int ns = n_seeds;
        if (mode == 0) sd = seeds + 5 * i;
        else if (multiseed_rule) { ns = or_multiseed_seeds(P, T[i], tbl); if (n_seeds > 0 && n_seeds < ns) ns = n_seeds; sd = tbl; }
        or_solve_point(P, n_nodes, pm, cm, wm, T[i], mu + 3 * i, xi[i], mode, ns, sd, o, &out[i]);
    }
}

int or_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int or_sizeof_result(void) { return (int)sizeof(or_result); }
int or_sizeof_opts(void) { return (int)sizeof(or_opts); }
int or_sizeof_params(void) { return (int)sizeof(or_params); }

/* ------------------------------------------------------------------------- */
/* K data of the relaxation-time chain: build_K_data                          */
/* (scripts/relaxtime/run_gap_transport_scan.jl:297-305)                      */
/* ------------------------------------------------------------------------- */
/* const_integral_term_A (OneLoopIntegrals.jl:507-517): int_0^Lambda p^2/E dp in closed form */
double or_const_integral_term_A(const or_params *P, double m) {
    const double L = P->Lambda;
    const double mp = m > 0.0 ? m : 0.0;
    if (mp < 1e-14) return L * L / 2.0;
    const double r = sqrt(L * L + mp * mp);
    return (L * r - mp * mp * log((L + r) / mp)) / 2.0;
}

/* A (OneLoopIntegrals.jl:531-543): 4 [ -const_integral_term_A(m)
 *   + sum_i w_i p_i^2 / E_i (f+(E_i) + f-(E_i)) ],  E = sqrt(p^2 + m^2), with the PNJL
 * distributions of QuarkDistribution.jl:14-51 (distribution_value, :14-61 of the same file) */
double or_one_loop_A(const or_params *P, int n_nodes, const double *p, const double *w, double m, double mu,
                     double T, double Phi, double Phib) {
    double integral = -or_const_integral_term_A(P, m);
    for (int i = 0; i < n_nodes; ++i) {
        const double E = sqrt(p[i] * p[i] + m * m);
        integral += w[i] * p[i] * p[i] / E * (quark_dist(E, mu, T, Phi, Phib) + antiquark_dist(E, mu, T, Phi, Phib));
    }
    return 4.0 * integral;
}

/* calculate_effective_couplings (EffectiveCouplings.jl:242-279) with
 * coupling_matrix_determinant (:112-115): out[12] = K0+, K0-, K123+, K123-, K4567+, K4567-,
 * K8+, K8-, K08+, K08-, det K+, det K- */
void or_effective_couplings(double G, double K, double Gu, double Gs, double *out) {
    const double t0 = (1.0 / 3.0) * K * (2.0 * Gu + Gs);
    const double t123 = 0.5 * K * Gs;
    const double t4567 = 0.5 * K * Gu;
    const double t8 = (1.0 / 6.0) * K * (4.0 * Gu - Gs);
    const double t08 = (1.0 / 6.0) * sqrt(2.0) * K * (Gu - Gs);
    const double K0p = G - t0, K0m = G + t0, K8p = G + t8, K8m = G - t8, K08p = t08, K08m = -t08;
    out[0] = K0p; out[1] = K0m;
    out[2] = G + t123; out[3] = G - t123;
    out[4] = G + t4567; out[5] = G - t4567;
    out[6] = K8p; out[7] = K8m;
    out[8] = K08p; out[9] = K08m;
    out[10] = K0p * K8p - K08p * K08p;
    out[11] = K0m * K8m - K08m * K08m;
}

/* build_K_data for one point: out[17] = A_u, A_d, A_s, G_u, G_s, then the 12 couplings of
 * or_effective_couplings.  A_d = A_u as build_K_data sets it; G^f = -N_c/(4 pi^2) m_f A_f
 * (calculate_G_from_A, EffectiveCouplings.jl:56-60, N_c = 3).  mu_u / mu_s: the reference
 * passes one quark chemical potential for both. */
void or_kdata(const or_params *P, int n_nodes, const double *p, const double *w, double T, double mu_u, double mu_s,
              double m_u, double m_s, double Phi, double Phib, double *out) {
    const double pi = 3.14159265358979323846;
    const double Au = or_one_loop_A(P, n_nodes, p, w, m_u, mu_u, T, Phi, Phib);
    const double As = or_one_loop_A(P, n_nodes, p, w, m_s, mu_s, T, Phi, Phib);
    const double Nc = 3.0;
    out[0] = Au; out[1] = Au; out[2] = As;
    out[3] = -Nc / (4.0 * pi * pi) * (m_u * Au);
    out[4] = -Nc / (4.0 * pi * pi) * (m_s * As);
    or_effective_couplings(P->G, P->K, out[3], out[4], out + 5);
}

/* ------------------------------------------------------------------------- */
/* Implicit derivatives: ThermoDerivatives.jl (mass_derivatives :132-173,     */
/* thermo_derivatives :184-249, bulk_viscosity_coefficients :342-465)          */
/* ------------------------------------------------------------------------- */
/* The reference differentiates the solution x(theta) of F(x; theta) = 0, theta = (T, mu)
 * with every mu_f shifted together, by the implicit function theorem
 * (ImplicitDifferentiation.jl: dx/dtheta = -(dF/dx)^-1 dF/dtheta) and ForwardDiff through
 * calculate_thermo / calculate_rho.  Restated here with a second-order jet in the seven
 * variables (phi_u, phi_d, phi_s, Phi, Phibar, T, mu): one jet evaluation of Omega gives every
 * first and second derivative the chain rule needs, exactly as nested forward-mode AD does. */
#define NV7 7
#define NH7 28
static int HI7[NH7], HJ7[NH7];
static void init_h7(void) {
    static int done = 0;
    if (done) return;
    int k = 0;
    for (int i = 0; i < NV7; ++i)
        for (int j = i; j < NV7; ++j) { HI7[k] = i; HJ7[k] = j; ++k; }
    done = 1;
}
static int h7(int i, int j) { /* index of (i, j) in the packed upper triangle */
    if (i > j) { int t = i; i = j; j = t; }
    return i * NV7 - i * (i - 1) / 2 + (j - i);
}
typedef struct { double v, g[NV7], h[NH7]; } jet7;
static jet7 k_const(double c) { jet7 r; memset(&r, 0, sizeof r); r.v = c; return r; }
static jet7 k_var(double c, int i) { jet7 r = k_const(c); r.g[i] = 1.0; return r; }
static jet7 k_add(jet7 a, jet7 b) {
    jet7 r; r.v = a.v + b.v;
    for (int i = 0; i < NV7; ++i) r.g[i] = a.g[i] + b.g[i];
    for (int k = 0; k < NH7; ++k) r.h[k] = a.h[k] + b.h[k];
    return r;
}
static jet7 k_scale(jet7 a, double c) {
    jet7 r; r.v = a.v * c;
    for (int i = 0; i < NV7; ++i) r.g[i] = a.g[i] * c;
    for (int k = 0; k < NH7; ++k) r.h[k] = a.h[k] * c;
    return r;
}
static jet7 k_sub(jet7 a, jet7 b) { return k_add(a, k_scale(b, -1.0)); }
static jet7 k_addc(jet7 a, double c) { a.v += c; return a; }
static jet7 k_mul(jet7 a, jet7 b) {
    jet7 r; r.v = a.v * b.v;
    for (int i = 0; i < NV7; ++i) r.g[i] = a.v * b.g[i] + b.v * a.g[i];
    for (int k = 0; k < NH7; ++k)
        r.h[k] = a.v * b.h[k] + b.v * a.h[k] + a.g[HI7[k]] * b.g[HJ7[k]] + a.g[HJ7[k]] * b.g[HI7[k]];
    return r;
}
static jet7 k_fn(jet7 a, double f0, double f1, double f2) {
    jet7 r; r.v = f0;
    for (int i = 0; i < NV7; ++i) r.g[i] = f1 * a.g[i];
    for (int k = 0; k < NH7; ++k) r.h[k] = f1 * a.h[k] + f2 * a.g[HI7[k]] * a.g[HJ7[k]];
    return r;
}
static jet7 k_exp(jet7 a) { double e = exp(a.v); return k_fn(a, e, e, e); }
static jet7 k_log(jet7 a) { double i = 1.0 / a.v; return k_fn(a, log(a.v), i, -i * i); }
static jet7 k_sqrt(jet7 a) { double s = sqrt(a.v), d1 = 1.0 / (2.0 * s); return k_fn(a, s, d1, -d1 / (2.0 * a.v)); }
static jet7 k_inv(jet7 a) { double i = 1.0 / a.v; return k_fn(a, i, -i * i, 2.0 * i * i * i); }
static jet7 k_abs(jet7 a) { return signbit(a.v) ? k_scale(a, -1.0) : a; }
static jet7 k_maxc(jet7 a, double c) { return (a.v < c) ? k_const(c) : a; }

/* Integrals.jl:193-238 calculate_log_term with E, mu, T, Phi, Phibar all jets */
static jet7 log_term_jet7(jet7 E, jet7 mu, jet7 T, jet7 Phi, jet7 Phib) {
    jet7 invT = k_inv(T);
    jet7 a = k_scale(k_mul(k_sub(E, mu), invT), -1.0);
    jet7 b = k_scale(k_mul(k_add(E, mu), invT), -1.0);
    jet7 tP = k_scale(Phi, 3.0), tPb = k_scale(Phib, 3.0), lfp, lfm;
    if (a.v > 0) {
        jet7 e1 = k_exp(k_scale(a, -2.0)), e2 = k_exp(k_scale(a, -1.0)), e0 = k_exp(k_scale(a, -3.0));
        jet7 term = k_addc(k_add(k_add(e0, k_mul(tP, e1)), k_mul(tPb, e2)), 1.0);
        lfp = k_add(k_scale(a, 3.0), k_log(k_maxc(term, POLYAKOV_EPS)));
    } else {
        jet7 e1 = k_exp(a), e2 = k_mul(e1, e1), e3 = k_mul(e1, e2);
        jet7 f = k_add(k_add(k_addc(k_mul(tP, e1), 1.0), k_mul(tPb, e2)), e3);
        lfp = k_log(k_maxc(f, POLYAKOV_EPS));
    }
    if (b.v > 0) {
        jet7 e1 = k_exp(k_scale(b, -2.0)), e2 = k_exp(k_scale(b, -1.0)), e0 = k_exp(k_scale(b, -3.0));
        jet7 term = k_addc(k_add(k_add(e0, k_mul(tPb, e1)), k_mul(tP, e2)), 1.0);
        lfm = k_add(k_scale(b, 3.0), k_log(k_maxc(term, POLYAKOV_EPS)));
    } else {
        jet7 e1 = k_exp(b), e2 = k_mul(e1, e1), e3 = k_mul(e1, e2);
        jet7 f = k_add(k_add(k_addc(k_mul(tPb, e1), 1.0), k_mul(tP, e2)), e3);
        lfm = k_log(k_maxc(f, POLYAKOV_EPS));
    }
    return k_add(lfp, lfm);
}

/* calculate_omega (Thermodynamics.jl:181-195) with x, T and the common mu shift as jets:
 * mu_f = mu0_f + s, s = 0 the seventh variable. */
static jet7 omega_jet7(const or_params *P, const or_nodes *nd, const double *xv, const double *mu0, double T0v,
                       double xi) {
    init_h7();
    jet7 x[5];
    for (int i = 0; i < 5; ++i) x[i] = k_var(xv[i], i);
    jet7 T = k_var(T0v, 5), s = k_var(0.0, 6);
    jet7 sq = k_add(k_add(k_mul(x[0], x[0]), k_mul(x[1], x[1])), k_mul(x[2], x[2]));
    jet7 chi = k_sub(k_scale(sq, 2.0 * P->G), k_scale(k_mul(k_mul(x[0], x[1]), x[2]), 4.0 * P->K));
    /* U (Thermodynamics.jl:124-130), T a jet */
    jet7 r = k_scale(k_inv(T), P->T0);
    jet7 Ta = k_addc(k_add(k_scale(r, P->a1), k_scale(k_mul(r, r), P->a2)), P->a0);
    jet7 Tb = k_scale(k_mul(k_mul(r, r), r), P->b3);
    jet7 pp = k_mul(x[4], x[3]);
    jet7 cub = k_add(k_mul(k_mul(x[4], x[4]), x[4]), k_mul(k_mul(x[3], x[3]), x[3]));
    jet7 val = k_sub(k_add(k_addc(k_scale(pp, -6.0), 1.0), k_scale(cub, 4.0)), k_scale(k_mul(pp, pp), 3.0));
    jet7 lg = (val.v <= 0 || val.v < POLYAKOV_EPS) ? k_const(log(POLYAKOV_EPS)) : k_log(val);
    jet7 T2 = k_mul(T, T), T4 = k_mul(T2, T2);
    jet7 U = k_mul(T4, k_add(k_mul(k_scale(Ta, -0.5), pp), k_mul(Tb, lg)));
    /* masses and vacuum term (Integrals.jl:123-145) */
    jet7 M[3];
    M[0] = k_add(k_addc(k_scale(x[0], -4.0 * P->G), P->m_ud0), k_mul(k_scale(x[1], 2.0 * P->K), x[2]));
    M[1] = k_add(k_addc(k_scale(x[1], -4.0 * P->G), P->m_ud0), k_mul(k_scale(x[0], 2.0 * P->K), x[2]));
    M[2] = k_add(k_addc(k_scale(x[2], -4.0 * P->G), P->m_s0), k_mul(k_scale(x[0], 2.0 * P->K), x[1]));
    jet7 vac = k_const(0.0);
    const double L = P->Lambda;
    for (int f = 0; f < 3; ++f) {
        jet7 ms = k_addc(k_abs(M[f]), 1e-12);
        jet7 ms2 = k_mul(ms, ms);
        jet7 sqv = k_sqrt(k_addc(ms2, L * L));
        jet7 poly = k_mul(k_scale(sqv, L), k_addc(ms2, 2.0 * L * L));
        jet7 lt = k_mul(k_mul(ms2, ms2), k_log(k_mul(k_addc(sqv, L), k_inv(ms))));
        vac = k_add(vac, k_scale(k_sub(poly, lt), 1.0 / (16.0 * M_PI * M_PI)));
    }
    jet7 esum = k_scale(vac, -2.0 * P->N_color);
    /* Integrals.jl:248-259 */
    jet7 total = k_const(0.0);
    for (int f = 0; f < 3; ++f) {
        jet7 M2 = k_mul(M[f], M[f]);
        jet7 muf = k_addc(s, mu0[f]);
        for (int k = 0; k < nd->n; ++k) {
            const double p = nd->p[k], c = nd->c[k], pc = p * c;
            jet7 E = k_sqrt(k_addc(M2, p * p + xi * (pc * pc)));
            total = k_add(total, k_scale(log_term_jet7(E, muf, T, x[3], x[4]), nd->w[k]));
        }
    }
    jet7 logsum = k_mul(k_scale(T, -2.0), total);
    return k_add(k_add(k_add(chi, U), esum), logsum);
}

/* Derivatives of a solved state x at (T, mu_f), theta = (T, mu) with every mu_f moved together.
 * out (OR_NDERIV doubles):
 *   [0..4]  dx/dT            [5..9]  dx/dmu
 *   [10..12] dM/dT           [13..15] dM/dmu
 *   16 s = -dOmega/dT        17 n_B = -(1/3) dOmega/dmu (sum of rho_f / 3)
 *   18 ds/dT  19 ds/dmu      20 dn_B/dT  21 dn_B/dmu     (total, through x(theta))
 *   22 P      23 dP/dT       24 dP/dmu
 *   25 eps = -P + 3 mu_mean n_B ... (below)  26 deps/dT  27 deps/dmu
 *   28 dP/deps|n             29 dP/dn|eps                (thermo_derivatives :225-229)
 *   30 v_n^2                 31 dmu_B/dT|sigma           (bulk_viscosity_coefficients :440-457)
 * eps = -P + sum_f mu_f rho_f + T s (calculate_thermo, Thermodynamics.jl:233-244); the chain
 * rule for it uses d(sum mu_f rho_f)/dtheta = sum_f mu_f drho_f/dtheta + [theta = mu] sum rho_f.
 * Returns 0, or 1 when the Hessian is singular. */
#define OR_NDERIV 32
int or_thermo_derivs(const or_params *P, int n_nodes, const double *pm, const double *cm, const double *wm,
                     const double *x, const double *mu, double T, double xi, double *out) {
    or_nodes nd = {n_nodes, pm, cm, wm};
    jet7 om = omega_jet7(P, &nd, x, mu, T, xi);
    double H[25], rhsT[5], rhsM[5], dxT[5], dxM[5];
    for (int i = 0; i < 5; ++i) {
        for (int j = 0; j < 5; ++j) H[i * 5 + j] = om.h[h7(i, j)];
        rhsT[i] = -om.h[h7(i, 5)];
        rhsM[i] = -om.h[h7(i, 6)];
    }
    if (lu_solve(5, H, rhsT, dxT) != 0 || lu_solve(5, H, rhsM, dxM) != 0) return 1;
    for (int i = 0; i < 5; ++i) { out[i] = dxT[i]; out[5 + i] = dxM[i]; }
    /* dM/dtheta = dM/dx . dx/dtheta (Thermodynamics.jl:81-90) */
    const double G4 = 4.0 * P->G, K2 = 2.0 * P->K;
    const double Jm[3][3] = {{-G4, K2 * x[2], K2 * x[1]}, {K2 * x[2], -G4, K2 * x[0]}, {K2 * x[1], K2 * x[0], -G4}};
    for (int f = 0; f < 3; ++f) {
        double a = 0.0, b = 0.0;
        for (int k = 0; k < 3; ++k) { a += Jm[f][k] * dxT[k]; b += Jm[f][k] * dxM[k]; }
        out[10 + f] = a;
        out[13 + f] = b;
    }
    /* s = -Omega_T and 3 n_B = sum rho_f = -Omega_mu, and their total derivatives */
    const double OT = om.g[5], OM = om.g[6];
    double sT = -om.h[h7(5, 5)], sM = -om.h[h7(5, 6)], nT = -om.h[h7(5, 6)], nM = -om.h[h7(6, 6)];
    double PT = -OT, PM = -OM;
    for (int i = 0; i < 5; ++i) {
        sT -= om.h[h7(5, i)] * dxT[i];
        sM -= om.h[h7(5, i)] * dxM[i];
        nT -= om.h[h7(6, i)] * dxT[i];
        nM -= om.h[h7(6, i)] * dxM[i];
        PT -= om.g[i] * dxT[i];
        PM -= om.g[i] * dxM[i];
    }
    const double s = -OT, nB = -OM / 3.0;
    nT /= 3.0;
    nM /= 3.0;
    out[16] = s; out[17] = nB; out[18] = sT; out[19] = sM; out[20] = nT; out[21] = nM;
    /* P and eps (calculate_thermo) with rho_f = -dOmega/dmu_f at fixed x: sum_f mu_f rho_f needs
     * the per-flavour densities; with every mu_f moved together d(mu_f)/dmu = 1 */
    double rho[3], murho = 0.0;
    {
        or_thermo th;
        or_thermo_eval(P, n_nodes, pm, cm, wm, x, mu, T, xi, &th);
        for (int f = 0; f < 3; ++f) { rho[f] = th.rho[f]; murho += mu[f] * rho[f]; }
    }
    const double Pv = -om.v;
    /* d(sum mu_f rho_f)/dtheta: the per-flavour rho_f derivatives are not separated by the
     * shared-mu jet, so for mu_u = mu_d = mu_s = mu it is mu * d(3 n_B)/dtheta (+ 3 n_B for
     * theta = mu); the reference's thermo_derivatives always has equal mu_f. */
    const double mubar = (mu[0] + mu[1] + mu[2]) / 3.0;
    const double eps = -Pv + murho + T * s;
    const double eT = -PT + mubar * 3.0 * nT + s + T * sT;
    const double eM = -PM + 3.0 * nB + mubar * 3.0 * nM + T * sM;
    out[22] = Pv; out[23] = PT; out[24] = PM; out[25] = eps; out[26] = eT; out[27] = eM;
    const double den_e = eT * nM - eM * nT, den_n = nT * eM - nM * eT;
    out[28] = den_e == 0 ? NAN : (PT * nM - PM * nT) / den_e;
    out[29] = den_n == 0 ? NAN : (PT * eM - PM * eT) / den_n;
    /* bulk_viscosity_coefficients: mu_B = 3 mu_q */
    const double sMB = sM / 3.0, nMB = nM / 3.0;
    out[30] = (s * nMB - nB * nT) / (T * (sT * nMB - sMB * nT));
    out[31] = -(nB * sT - s * nT) / (nB * sMB - s * nMB);
    return 0;
}
