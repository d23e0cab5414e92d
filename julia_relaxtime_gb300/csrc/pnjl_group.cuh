// pnjl_group.cuh -- the per-task solver of libpnjl_cuda: a group of G lanes (G = 32, one
// warp) that runs NLsolve-style Newton and trust-region solves of one (point, seed) on top of
// the node passes of pnjl_solver.cuh, plus the helpers the solve kernels share (node-table
// staging, candidate records, output writing).  Included by the kernel translation units.
#pragma once

#include "pnjl_kernels.h"
#include "pnjl_solver.cuh"

namespace pnjl {

// ---------------------------------------------------------------------------------------
// Stage the separable node tables (a few KB) into shared memory.
__device__ __forceinline__ NodeView stage_nodes(const KernelNodes &kn, void *smem) {
    NodeView nv;
    nv.p_num = kn.p_num;
    nv.t_num = kn.t_num;
    const int np = kn.p_num, nt = kn.t_num;
    double *sd = (double *)smem;
    for (int i = threadIdx.x; i < np; i += blockDim.x) { sd[i] = kn.p2[i]; sd[np + i] = kn.A[i]; }
    for (int i = threadIdx.x; i < nt; i += blockDim.x) { sd[2 * np + i] = kn.c2[i]; sd[2 * np + nt + i] = kn.B[i]; }
    float *sf = (float *)(sd + 2 * (np + nt));
    for (int i = threadIdx.x; i < np; i += blockDim.x) { sf[i] = kn.p2f[i]; sf[np + i] = kn.Af[i]; }
    for (int i = threadIdx.x; i < nt; i += blockDim.x) { sf[2 * np + i] = kn.c2f[i]; sf[2 * np + nt + i] = kn.Bf[i]; }
    nv.p2 = sd; nv.A = sd + np; nv.c2 = sd + 2 * np; nv.B = sd + 2 * np + nt;
    nv.p2f = sf; nv.Af = sf + np; nv.c2f = sf + 2 * np; nv.Bf = sf + 2 * np + nt;
    nv.p2l = nv.Al = nv.c2l = nv.Bl = nullptr;
    nv.expt = nullptr;
    nv.exp64 = nullptr;
    if (kn.lo && kn.expt) {
        const int m = 2 * (np + nt);
        float *sl = sf + m;
        for (int i = threadIdx.x; i < m; i += blockDim.x) sl[i] = kn.lo[i];
        float *se = sl + m;
        for (int i = threadIdx.x; i < kExpTableFloats; i += blockDim.x) se[i] = kn.expt[i];
        nv.p2l = sl; nv.Al = sl + np; nv.c2l = sl + 2 * np; nv.Bl = sl + 2 * np + nt;
        nv.expt = se;
        nv.exp64 = (const double *)(se + kExp64Offset);
    }
    return nv;
}


struct Counters {
    int64_t v[kStatCount];
};

__device__ __forceinline__ double qnan() { return __longlong_as_double(0x7ff8000000000000ll); }

__device__ __forceinline__ bool same_root(const double *x, const double *y);

// The plateau bound of a slot that has no per-point root (MultiSeed table and fallback
// mode): the Omega of the slot's seed 0 once that seed is certified usable.  Seeds s > 0 wait
// for seed 0's verdict (bounded by `polls` sleeps of 128 ns; a wait that runs out is counted
// and leaves the seed without a bound) only when their Newton refinement reaches a plateau,
// on the warp that runs the task.  Seed 0 waits for no later seed, and its task was taken
// before theirs (tasks are taken in order) by a warp that runs it to its end or queues its
// certification for the certifying warps, which never wait here; so every wait ends.  The
// bound is fixed per slot: what it drops does not depend on timing.
struct Anchor {
    const int *state;      // the slot's anchor_state
    const double *omega;   // the slot's anchor_omega
    unsigned polls;
};
constexpr unsigned kAnchorSleepNs = 128;

template <int G>
struct Group {
    const DevParams &P;
    const NodeView &nv;
    int gl;
    unsigned mask;
    Counters &cnt;

    __device__ __forceinline__ int leader() const { return (int)(threadIdx.x & 31) & ~(G - 1); }

    // Isospin symmetry: with mu_u == mu_d and phi_u == phi_d the exact Newton (or dogleg) step
    // has p_u == p_d; the 5x5 elimination leaves them unequal in the last bit.  Projecting the
    // step keeps the state symmetric, so every pass evaluates the u and d flavours once.
    __device__ static __forceinline__ void symmetrize_step(const PointIn &pt, const double *x, double *p) {
        if (pt.mu[0] == pt.mu[1] && x[0] == x[1]) {
            const double m = 0.5 * (p[0] + p[1]);
            p[0] = m;
            p[1] = m;
        }
    }

    // residual and Jacobian at x (one Newton pass)
    __device__ __noinline__ void eval_newton(const PointIn &pt, const double *x, double *F, double *J) {
        double M[3];
        masses(P, x, M);
        PassSums S;
        node_pass<double, false, true, true, false, G>(nv, pt, x, M, gl, mask, S, cnt.v[kStatEvalsNewton64]);
        Eval ev;
        double V, V1[3], V2[3];
        vacuum_terms<G>(P, M, gl, mask, leader(), V, V1, V2);
        assemble<true, true, false>(P, pt, x, M, S, V, V1, V2, ev);
        for (int i = 0; i < 5; ++i) F[i] = ev.F[i];
        for (int i = 0; i < 25; ++i) J[i] = ev.J[i];
        cnt.v[kStatPasses64] += 1;
    }

    // Omega, entropy, rho_f and number densities at x (one thermo pass) -> candidate fields
    // det5_negative of the FP64 Jacobian at x (a root of the FP64 path, which keeps no
    // Jacobian with its candidate): one FP64 Newton pass.
    __device__ bool unstable_root(const PointIn &pt, const double *x) {
        double F[5], J[25];
        eval_newton(pt, x, F, J);
        return det5_negative(J);
    }

    __device__ __noinline__ void eval_thermo(const PointIn &pt, const SolveOpts &o, Candidate &c) {
        double M[3];
        masses(P, c.x, M);
        PassSums S;
        node_pass<double, false, false, false, true, G>(nv, pt, c.x, M, gl, mask, S, cnt.v[kStatEvalsThermo64]);
        Eval ev;
        double V, V1[3], V2[3];
        vacuum_terms<G>(P, M, gl, mask, leader(), V, V1, V2);
        assemble<false, false, true>(P, pt, c.x, M, S, V, V1, V2, ev);
        cnt.v[kStatPasses64] += 1;
        postprocess(P, pt, o, ev, c);
    }

    // NLsolve :newton (static line search) from x0
    __device__ void newton(const PointIn &pt, const double *x0, const SolveOpts &o, Candidate &c, int max_iter = -1) {
        if (max_iter < 0) max_iter = o.max_iter;
        double x[5], xold[5], p[5], F[5], J[25];
#pragma unroll
        for (int i = 0; i < 5; ++i) { x[i] = x0[i]; xold[i] = qnan(); }
        eval_newton(pt, x, F, J);
        c.exception = !all_finite5(F);
        if (c.exception) {
            for (int i = 0; i < 5; ++i) c.x[i] = x0[i];
            c.residual_norm = qnan();
            c.iterations = 0;
            c.f_converged = false;
            c.phys = false;
            return;
        }
        int it = 0;
        bool xconv = false, fconv = norm_inf5(F) < o.ftol;
        bool stopped = any_nan5(x) || any_nan5(F);
        bool converged = fconv;
        while (!stopped && !converged && it < max_iter) {
            ++it;
            if (lu_solve5(J, F, p)) {
#pragma unroll
                for (int i = 0; i < 5; ++i) p[i] = -p[i];
            } else {
                levenberg_step(J, F, p);
            }
            symmetrize_step(pt, x, p);
#pragma unroll
            for (int i = 0; i < 5; ++i) { xold[i] = x[i]; x[i] += p[i]; }
            eval_newton(pt, x, F, J);
            double dx = 0.0;
            bool dxn = false;
#pragma unroll
            for (int i = 0; i < 5; ++i) {
                const double d = fabs(x[i] - xold[i]);
                dxn |= isnan(d);
                dx = d > dx ? d : dx;
            }
            xconv = !any_nan5(xold) && !dxn && dx < o.xtol;
            fconv = norm_inf5(F) < o.ftol;
            stopped = any_nan5(x) || any_nan5(F);
            converged = xconv || fconv;
        }
        for (int i = 0; i < 5; ++i) c.x[i] = x[i];
        c.residual_norm = norm_inf5(F);
        c.iterations = it;
        c.f_converged = fconv;
        eval_thermo(pt, o, c);
    }

    // singular Jacobian: p = -(J'J + lambda I) \ J'F, lambda = 1e6 sqrt(n eps) sum|J'J|
    __device__ static void levenberg_step(const double *J, const double *F, double *p) {
        double g[5], A[25], s = 0.0;
        for (int i = 0; i < 5; ++i) {
            double a = 0.0;
            for (int k = 0; k < 5; ++k) a += J[k * 5 + i] * F[k];
            g[i] = a;
        }
        for (int i = 0; i < 5; ++i)
            for (int j = 0; j < 5; ++j) {
                double a = 0.0;
                for (int k = 0; k < 5; ++k) a += J[k * 5 + i] * J[k * 5 + j];
                A[i * 5 + j] = -a;
                s += fabs(a);
            }
        const double lambda = 1e6 * sqrt(5.0 * 2.220446049250313e-16) * s;
        for (int i = 0; i < 5; ++i) A[i * 5 + i] -= lambda;
        if (!lu_solve5(A, g, p))
            for (int i = 0; i < 5; ++i) p[i] = qnan();
    }

    // NLsolve :trust_region (dogleg, autoscale) from x0
    __device__ void trust_region(const PointIn &pt, const double *x0, const SolveOpts &o, Candidate &c) {
        double x[5], xold[5], d[5], p[5], r[5], Jacc[25], F[5], J[25];
        for (int i = 0; i < 5; ++i) { x[i] = x0[i]; xold[i] = qnan(); }
        eval_newton(pt, x, r, Jacc);
        cnt.v[kStatTrRuns] += 1;
        c.exception = !all_finite5(r);
        if (c.exception) {
            for (int i = 0; i < 5; ++i) c.x[i] = x0[i];
            c.residual_norm = qnan();
            c.iterations = 0; c.f_converged = false; c.phys = false;
            return;
        }
        int it = 0;
        bool fconv = norm_inf5(r) < o.ftol;
        bool stopped = any_nan5(x) || any_nan5(r);
        bool converged = fconv;
        if (!converged) {
            for (int j = 0; j < 5; ++j) {
                double s = 0.0;
                for (int i = 0; i < 5; ++i) s += Jacc[i * 5 + j] * Jacc[i * 5 + j];
                d[j] = sqrt(s);
                if (d[j] == 0.0) d[j] = 1.0;
            }
            double delta = 0.0;
            for (int i = 0; i < 5; ++i) delta += (d[i] * x[i]) * (d[i] * x[i]);
            delta = sqrt(delta);
            if (delta == 0.0) delta = 1.0;
            while (!stopped && !converged && it < o.max_iter) {
                ++it;
                dogleg(p, r, d, Jacc, delta);
                symmetrize_step(pt, x, p);
                for (int i = 0; i < 5; ++i) { xold[i] = x[i]; x[i] += p[i]; }
                eval_newton(pt, x, F, J);
                double sr = 0.0, sf = 0.0, sp = 0.0;
                for (int k = 0; k < 5; ++k) {
                    double a = 0.0;
                    for (int i = 0; i < 5; ++i) a += Jacc[k * 5 + i] * p[i];
                    const double rp = a + r[k];
                    sr += r[k] * r[k];
                    sf += F[k] * F[k];
                    sp += rp * rp;
                }
                const double rho = (sr - sf) / (sr - sp);
                if (rho > 1e-4) {
                    for (int i = 0; i < 5; ++i) r[i] = F[i];
                    for (int i = 0; i < 25; ++i) Jacc[i] = J[i];
                    for (int j = 0; j < 5; ++j) {
                        double s = 0.0;
                        for (int i = 0; i < 5; ++i) s += Jacc[i * 5 + j] * Jacc[i * 5 + j];
                        const double cn = sqrt(s);
                        d[j] = (0.1 * d[j] > cn) ? 0.1 * d[j] : cn;
                    }
                    double dx = 0.0;
                    bool dxn = false;
                    for (int i = 0; i < 5; ++i) {
                        const double dd = fabs(x[i] - xold[i]);
                        dxn |= isnan(dd);
                        dx = dd > dx ? dd : dx;
                    }
                    const bool xconv = !dxn && dx < o.xtol;
                    fconv = norm_inf5(r) < o.ftol;
                    converged = xconv || fconv;
                } else {
                    for (int i = 0; i < 5; ++i) x[i] -= p[i];
                    converged = false;
                }
                double wp = 0.0;
                for (int i = 0; i < 5; ++i) wp += (d[i] * p[i]) * (d[i] * p[i]);
                wp = sqrt(wp);
                if (rho < 0.1) delta = delta / 2.0;
                else if (rho >= 0.9) delta = 2.0 * wp;
                else if (rho >= 0.5) delta = fmax(delta, 2.0 * wp);
                stopped = any_nan5(x) || any_nan5(F);
            }
        }
        for (int i = 0; i < 5; ++i) c.x[i] = x[i];
        c.residual_norm = norm_inf5(r);
        c.iterations = it;
        c.f_converged = fconv;
        eval_thermo(pt, o, c);
    }

    // Powell dogleg inside ||D p|| <= delta (Nocedal & Wright, section 4.1)
    __device__ static void dogleg(double *p, const double *r, const double *d, const double *J, double delta) {
        double pi[5], pc[5], g[5];
        if (!lu_solve5(J, r, pi)) {
            double JJ[25], Jr[5];
            for (int i = 0; i < 5; ++i) {
                double a = 0.0;
                for (int k = 0; k < 5; ++k) a += J[k * 5 + i] * r[k];
                Jr[i] = a;
            }
            for (int i = 0; i < 5; ++i)
                for (int j = 0; j < 5; ++j) {
                    double a = 0.0;
                    for (int k = 0; k < 5; ++k) a += J[k * 5 + i] * J[k * 5 + j];
                    JJ[i * 5 + j] = a;
                }
            for (int i = 0; i < 5; ++i) JJ[i * 5 + i] += 2.220446049250313e-16 * (1.0 + JJ[i * 5 + i]);
            if (!lu_solve5(JJ, Jr, pi))
                for (int i = 0; i < 5; ++i) pi[i] = 0.0;
        }
        for (int i = 0; i < 5; ++i) pi[i] = -pi[i];
        double wpi = 0.0;
        for (int i = 0; i < 5; ++i) wpi += (d[i] * pi[i]) * (d[i] * pi[i]);
        if (sqrt(wpi) <= delta) {
            for (int i = 0; i < 5; ++i) p[i] = pi[i];
            return;
        }
        for (int i = 0; i < 5; ++i) {
            double a = 0.0;
            for (int k = 0; k < 5; ++k) a += J[k * 5 + i] * r[k];
            g[i] = a / (d[i] * d[i]);
        }
        double Jg2 = 0.0, wg = 0.0;
        for (int k = 0; k < 5; ++k) {
            double a = 0.0;
            for (int i = 0; i < 5; ++i) a += J[k * 5 + i] * g[i];
            Jg2 += a * a;
        }
        for (int i = 0; i < 5; ++i) wg += (d[i] * g[i]) * (d[i] * g[i]);
        wg = sqrt(wg);
        for (int i = 0; i < 5; ++i) pc[i] = -(wg * wg) / Jg2 * g[i];
        double wpc = 0.0;
        for (int i = 0; i < 5; ++i) wpc += (d[i] * pc[i]) * (d[i] * pc[i]);
        wpc = sqrt(wpc);
        if (wpc >= delta) {
            for (int i = 0; i < 5; ++i) p[i] = g[i] * (-delta / wg);
            return;
        }
        double pd[5], bq = 0.0, aq = 0.0;
        for (int i = 0; i < 5; ++i) {
            pd[i] = pi[i] - pc[i];
            bq += (d[i] * pc[i]) * (d[i] * pd[i]);
            aq += (d[i] * pd[i]) * (d[i] * pd[i]);
        }
        bq *= 2.0;
        const double tau = (-bq + sqrt(bq * bq - 4.0 * aq * (wpc * wpc - delta * delta))) / (2.0 * aq);
        for (int i = 0; i < 5; ++i) p[i] = pc[i] + tau * pd[i];
    }

    // ---- mixed precision ---------------------------------------------------------------
    // Newton passes with the FP32 Kahan-compensated integrand (the 5x5 solve and the update
    // stay FP64), then FP64 refinement steps x <- x - J32^{-1} F64(x) until the FP64 residual
    // ||grad_x Omega||_inf is below ftol; Omega and the thermo output come from FP64 passes.
    static constexpr double kFtol32 = 1e-8;   // FP32 residual that ends the FP32 phase
    static constexpr double kStall32 = 1e-6;  // ... or a relative step this small ...
    static constexpr double kNoise32 = 1e-5;  // ... with the FP32 residual near its noise floor
    static constexpr double kLoose32 = 1e-3;  // residual at the iteration limit still handed on

    __device__ __noinline__ void eval_newton32(const PointIn &pt, const double *x, double *F, double *J) {
        double M[3];
        masses(P, x, M);
        PassSums S;
        node_pass_newton32<G>(nv, pt, x, M, gl, mask, S, cnt.v[kStatEvals32]);
        Eval ev;
        double V, V1[3], V2[3];
        vacuum_terms<G>(P, M, gl, mask, leader(), V, V1, V2);
        assemble<true, true, false, true>(P, pt, x, M, S, V, V1, V2, ev);
        for (int i = 0; i < 5; ++i) F[i] = ev.F[i];
        for (int i = 0; i < 25; ++i) J[i] = ev.J[i];
        cnt.v[kStatPasses32] += 1;
    }

    // Omega and the residual norm at x from one FP32 Kahan-compensated pass (FP64 vacuum, chi
    // and U terms): Omega accurate to ~1e-6 absolute, used only to discard candidates that
    // cannot win.
    __device__ __noinline__ double eval_omega32(const PointIn &pt, const double *x, double &fres) {
        double M[3];
        masses(P, x, M);
        PassSums S;
        node_pass<float, true, true, false, true, G>(nv, pt, x, M, gl, mask, S, cnt.v[kStatEvalsThermo32]);
        Eval ev;
        double V, V1[3], V2[3];
        vacuum_terms<G>(P, M, gl, mask, leader(), V, V1, V2);
        assemble<true, false, true>(P, pt, x, M, S, V, V1, V2, ev);
        cnt.v[kStatPasses32] += 1;
        fres = norm_inf5(ev.F);
        return ev.omega;
    }

    // Whether the FP32 root x32 cannot win the min-Omega selection against a certified
    // candidate of the same point with Omega `bound`.  The FP32 Omega pass is accurate to
    // ~1e-5 |Omega| (Kahan sums of FP32 terms).  A tight FP32 root (residual <= 1e-6) lies so
    // close to its FP64 root that their Omega differ by far less, so it is discarded when its
    // FP32 Omega exceeds bound by 1e-4 |bound|.  Loose end points of the FP32 phase (slow
    // convergence) are never discarded: refinement can still carry them far.  Anything not
    // discarded is refined and compared in FP64 as usual.
    static constexpr double kPruneTight = 1e-6, kPruneTightRtol = 1e-4;
    __device__ bool cannot_win(const PointIn &pt, const double *x32, double bound) {
        if (!(bound == bound)) return false;
        double fres = 0.0;
        const double om = eval_omega32(pt, x32, fres);
        const bool out = fres <= kPruneTight && om > bound + kPruneTightRtol * fmax(fabs(bound), 1.0);
        if (out) cnt.v[kStatPruned] += 1;
        return out;
    }

    // Residual at x from the float-float pass (FP32 pipe, ~1e-12 accurate); false when the
    // float-float tables are not staged or a sum is not finite (FP32 range exceeded).
    // The float-float residual pass, with or without the thermo sums: one compiled loop for
    // both (the two run back to back on every point, and one loop body keeps the instruction
    // cache of an SM sub-partition freer for the other warps' loops).
    __device__ __noinline__ void ff_pass_grad(const PointIn &pt, const double *x, const double *M, PassSums &S,
                                              bool thermo, int64_t &evals) {
        node_pass_ff<G, true, true>(nv, pt, x, M, gl, mask, S, evals, thermo);
    }

    __device__ __noinline__ bool eval_grad_ff(const PointIn &pt, const double *x, double *F) {
        if (!nv.p2l) return false;
        double M[3];
        masses(P, x, M);
        PassSums S;
        ff_pass_grad(pt, x, M, S, false, cnt.v[kStatEvalsFF]);
        Eval ev;
        double V, V1[3], V2[3];
        vacuum_terms<G>(P, M, gl, mask, leader(), V, V1, V2);
        assemble<true, false, false>(P, pt, x, M, S, V, V1, V2, ev);
        for (int i = 0; i < 5; ++i) F[i] = ev.F[i];
        cnt.v[kStatPasses32] += 1;
        return all_finite5(F);
    }

    // Residual and Jacobian at x from the float-float Newton pass (~1e-12 accurate, FP32
    // pipe); false when the tables are not staged or a value is not finite.
    __device__ __noinline__ bool eval_newton_ff(const PointIn &pt, const double *x, double *F, double *J) {
        if (!nv.p2l) return false;
        double M[3];
        masses(P, x, M);
        PassSums S;
        node_pass_ff<G, true, false, true>(nv, pt, x, M, gl, mask, S, cnt.v[kStatEvalsFF]);
        Eval ev;
        double V, V1[3], V2[3];
        vacuum_terms<G>(P, M, gl, mask, leader(), V, V1, V2);
        assemble<true, true, false>(P, pt, x, M, S, V, V1, V2, ev);
        bool ok = all_finite5(ev.F);
        for (int i = 0; i < 25; ++i) ok = ok && ev.J[i] == ev.J[i] && fabs(ev.J[i]) < 1e300;
        for (int i = 0; i < 5; ++i) F[i] = ev.F[i];
        for (int i = 0; i < 25; ++i) J[i] = ev.J[i];
        cnt.v[kStatPasses32] += 1;
        return ok;
    }

    // Residual at c.x and, from the same float-float pass, Omega, entropy, rho_f and the
    // number densities at c.x (the outputs should c.x be certified: the quantities the two
    // need per node -- E, the exponential, the Polyakov factors, n+ and n- -- are computed
    // once).  Bit 0 of the result: F finite; bit 1: the thermo fields of c were set (finite).
    __device__ __noinline__ int eval_grad_thermo_ff(const PointIn &pt, const SolveOpts &o, Candidate &c, double *F) {
        if (!nv.p2l) return 0;
        double M[3];
        masses(P, c.x, M);
        PassSums S;
        ff_pass_grad(pt, c.x, M, S, true, cnt.v[kStatEvalsFFGradThermo]);
        Eval ev;
        double V, V1[3], V2[3];
        vacuum_terms<G>(P, M, gl, mask, leader(), V, V1, V2);
        assemble<true, false, true>(P, pt, c.x, M, S, V, V1, V2, ev);
        cnt.v[kStatPasses32] += 1;
        for (int i = 0; i < 5; ++i) F[i] = ev.F[i];
        int r = all_finite5(F) ? 1 : 0;
        bool ok = ev.omega == ev.omega && fabs(ev.omega) < 1e300 && ev.dOdT == ev.dOdT;
        for (int f = 0; f < 3; ++f) ok = ok && ev.rho[f] == ev.rho[f] && ev.nq[f] == ev.nq[f] && ev.naq[f] == ev.naq[f];
        if (ok) {
            postprocess(P, pt, o, ev, c);
            r |= 2;
        }
        return r;
    }

    // Omega, entropy, rho_f and number densities at c.x from the float-float pass (the
    // outputs of a certified candidate, ~1e-13 relative); false when not available or not
    // finite (the caller then uses the FP64 thermo pass).
    __device__ __noinline__ bool eval_thermo_ff(const PointIn &pt, const SolveOpts &o, Candidate &c) {
        if (!nv.p2l) return false;
        double M[3];
        masses(P, c.x, M);
        PassSums S;
        node_pass_ff<G, false, true>(nv, pt, c.x, M, gl, mask, S, cnt.v[kStatEvalsFFThermo]);
        Eval ev;
        double V, V1[3], V2[3];
        vacuum_terms<G>(P, M, gl, mask, leader(), V, V1, V2);
        assemble<false, false, true>(P, pt, c.x, M, S, V, V1, V2, ev);
        cnt.v[kStatPasses32] += 1;
        bool ok = ev.omega == ev.omega && fabs(ev.omega) < 1e300 && ev.dOdT == ev.dOdT;
        for (int f = 0; f < 3; ++f) ok = ok && ev.rho[f] == ev.rho[f] && ev.nq[f] == ev.nq[f] && ev.naq[f] == ev.naq[f];
        if (!ok) return false;
        postprocess(P, pt, o, ev, c);
        return true;
    }

    // FP64 residual at x: the certification pass (node_pass_cert) where its table is staged.
    __device__ __noinline__ void eval_grad64(const PointIn &pt, const double *x, double *F) {
        double M[3];
        masses(P, x, M);
        PassSums S;
        if (nv.exp64) node_pass_cert<G>(nv, pt, x, M, gl, mask, S, cnt.v[kStatEvalsGrad64]);
        else node_pass<double, false, true, false, false, G>(nv, pt, x, M, gl, mask, S, cnt.v[kStatEvalsGrad64]);
        Eval ev;
        double V, V1[3], V2[3];
        vacuum_terms<G>(P, M, gl, mask, leader(), V, V1, V2);
        assemble<true, false, false>(P, pt, x, M, S, V, V1, V2, ev);
        for (int i = 0; i < 5; ++i) F[i] = ev.F[i];
        cnt.v[kStatPasses64] += 1;
    }

    // FP32-pass Newton from x0.  1: reached the FP32 floor, 0: did not converge, -1: residual
    // at x0 not finite.  The phase ends at the first of: a tiny residual; near the FP32 noise
    // floor (residual below kNoise32), a Newton step at the FP32 resolution (relative
    // kStall32) or a residual that stopped halving for two steps (the floor itself, or the
    // linear convergence of a nearly singular Jacobian, which the refinement then finishes);
    // the iteration limit, handed on only with a small residual.  Far from the floor the FP32
    // iteration goes on as the reference's FP64 Newton iteration would, within the same
    // iteration budget.  With `prior` (a certified root of the same point), an iterate that
    // comes within the duplicate tolerance of it ends the phase at once (1): it is inside that
    // root's Newton basin, and the seed is a duplicate of it (same_root), so the rest of its
    // iterations would be spent on a root already certified.
    __device__ int newton32(const PointIn &pt, const double *x0, const SolveOpts &o, double *x, double *J, int &iters,
                            const double *prior = nullptr) {
        double F[5], p[5];
        for (int i = 0; i < 5; ++i) x[i] = x0[i];
        eval_newton32(pt, x, F, J);
        iters = 0;
        if (!all_finite5(F)) return -1;
        int slow = 0;
        for (;;) {
            const double fn = norm_inf5(F);
            if (fn < kFtol32) return 1;
            if (iters >= o.max_iter) return fn < kLoose32 ? 1 : 0;
            if (lu_solve5<true>(J, F, p)) {
                for (int i = 0; i < 5; ++i) p[i] = -p[i];
            } else {
                levenberg_step(J, F, p);
            }
            symmetrize_step(pt, x, p);
            const double pn = norm_inf5(p), xn = norm_inf5(x);
            for (int i = 0; i < 5; ++i) x[i] += p[i];
            ++iters;
            if (prior && same_root(x, prior)) return 1;
            eval_newton32(pt, x, F, J);
            if (any_nan5(x) || any_nan5(F)) return 0;
            const double fnew = norm_inf5(F);
            if (fnew < kNoise32) {
                if (pn <= kStall32 * (1.0 + xn)) return 1;
                slow = fnew > 0.5 * fn ? slow + 1 : 0;
                if (slow >= 2) return 1;
            } else {
                slow = 0;
            }
        }
    }

    // NLsolve-style dogleg trust region on FP32 passes; same return codes and stop rules as
    // newton32, plus a trust radius collapsed to the FP32 resolution near the noise floor.
    __device__ int tr32(const PointIn &pt, const double *x0, const SolveOpts &o, double *x, double *Jacc, int &iters) {
        double d[5], p[5], r[5], F[5], J[25], xt[5];
        for (int i = 0; i < 5; ++i) x[i] = x0[i];
        eval_newton32(pt, x, r, Jacc);
        iters = 0;
        if (!all_finite5(r)) return -1;
        double fr = norm_inf5(r);
        if (fr < kFtol32) return 1;
        for (int j = 0; j < 5; ++j) {
            double s = 0.0;
            for (int i = 0; i < 5; ++i) s += Jacc[i * 5 + j] * Jacc[i * 5 + j];
            d[j] = sqrt(s);
            if (d[j] == 0.0) d[j] = 1.0;
        }
        double delta = 0.0;
        for (int i = 0; i < 5; ++i) delta += (d[i] * x[i]) * (d[i] * x[i]);
        delta = sqrt(delta);
        if (delta == 0.0) delta = 1.0;
        int slow = 0;
        while (iters < o.max_iter) {
            ++iters;
            dogleg(p, r, d, Jacc, delta);
            symmetrize_step(pt, x, p);
            for (int i = 0; i < 5; ++i) xt[i] = x[i] + p[i];
            eval_newton32(pt, xt, F, J);
            double sr = 0.0, sf = 0.0, sp = 0.0;
            for (int k = 0; k < 5; ++k) {
                double a = 0.0;
                for (int i = 0; i < 5; ++i) a += Jacc[k * 5 + i] * p[i];
                const double rp = a + r[k];
                sr += r[k] * r[k];
                sf += F[k] * F[k];
                sp += rp * rp;
            }
            const double rho = (sr - sf) / (sr - sp);
            double wp = 0.0;
            for (int i = 0; i < 5; ++i) wp += (d[i] * p[i]) * (d[i] * p[i]);
            wp = sqrt(wp);
            const double xn = norm_inf5(x);
            if (rho > 1e-4) {
                for (int i = 0; i < 5; ++i) { x[i] = xt[i]; r[i] = F[i]; }
                for (int i = 0; i < 25; ++i) Jacc[i] = J[i];
                for (int j = 0; j < 5; ++j) {
                    double s = 0.0;
                    for (int i = 0; i < 5; ++i) s += Jacc[i * 5 + j] * Jacc[i * 5 + j];
                    const double cn = sqrt(s);
                    d[j] = (0.1 * d[j] > cn) ? 0.1 * d[j] : cn;
                }
                const double fn = norm_inf5(r);
                if (any_nan5(x) || !(fn == fn)) return 0;
                if (fn < kFtol32) return 1;
                if (fn < kNoise32) {
                    if (norm_inf5(p) <= kStall32 * (1.0 + xn)) return 1;
                    slow = fn > 0.5 * fr ? slow + 1 : 0;
                    if (slow >= 2) return 1;
                } else {
                    slow = 0;
                }
                fr = fn;
            }
            if (rho < 0.1) delta = delta / 2.0;
            else if (rho >= 0.9) delta = 2.0 * wp;
            else if (rho >= 0.5) delta = fmax(delta, 2.0 * wp);
            if (fr < kNoise32 && delta <= kStall32 * (1.0 + xn)) return 1;
            if (!(delta > 0.0)) return 0;
        }
        return fr < kLoose32 ? 1 : 0;
    }

    // Seed 0's certified Omega for the plateau test of a slot without a per-point root (NaN:
    // seed 0 is not usable, or the wait ran out).
    __device__ double anchor_bound(const Anchor &an) {
        double b = qnan();
        if (gl == 0) {
            int st = *(volatile const int *)an.state;
            for (unsigned k = 0; st == 0 && k < an.polls; ++k) {
                __nanosleep(kAnchorSleepNs);
                st = *(volatile const int *)an.state;
            }
            if (st == 1) {
                __threadfence();
                b = __ldcg(an.omega);
            } else if (st == 0) {
                cnt.v[kStatWaitTimeouts] += 1;
            }
        }
        return __shfl_sync(mask, b, leader());
    }

    // Refinement and FP64 certification of an FP32 solution; fills c.
    // Steps x <- x - B^-1 F run on the FP32 pipe: F is the float-float residual (~1e-12
    // accurate), B starts as the FP32 Jacobian, gets Broyden's rank-one secant update
    // B <- B + (dF - B dx) dx' / (dx' dx) after every step, and is replaced by the float-float
    // Jacobian at x when the steps stop contracting (a slowly converging, nearly singular
    // root: Newton steps in float-float arithmetic, as accurate as FP64 Newton).  An FP64 residual pass is spent only
    // to certify: once the float-float residual is below ftol/10 (or has stopped decreasing
    // below ftol), and the root is accepted only when the FP64 residual ||grad_x Omega||_inf <
    // ftol.  Omega, entropy, rho_f and n_f at the certified state come from a float-float pass.
    // Without the float-float tables, or when their residuals are not finite, every residual is
    // FP64.  The seed's iteration budget (max_iter less the FP32 phase's iterations, as the
    // reference's NLsolve counts one budget per seed) bounds the steps; a seed that spends it
    // is not converged.  Steps that stop contracting even with fresh float-float Jacobians
    // hand the rest of the budget to newton_rescue from the best state.
    // The refinement stops at its first certification attempt and returns true: c.x is the
    // state to certify (certify(), at once or by a certifying warp), *th_out whether c's
    // thermo fields are those of c.x.  False: c is final; *th_out = -1 when the Omega prune
    // below dropped the seed (its Newton iteration converges, so, as in the reference, no
    // trust-region fallback follows), -2 / -3 for the give-up and plateau exits.
    // `bound` is the Omega of a certified candidate of the same point that this seed must
    // beat (NaN when there is none).  These tests drop a seed, not converged:
    // * Omega prune: a state reached by a contracting step (residual halved, now below 1e-5)
    //   whose float-float Omega -- computed at every step with the residual -- lies above the
    //   bound by more than 1e-9 |bound| plus 20 |F|inf |p|inf (p the last step): Newton's
    //   remaining path to the root is at most a few such steps long, |grad Omega| below |F|
    //   on it, so the root's Omega stays above the bound.  This drops the metastable roots of
    //   verification seeds before their FP64 certification.
    // * Plateau: float-float Newton steps with fresh float-float Jacobians have twice in a row
    //   failed to halve a residual still above 1e3 ftol.  Such a state is a spinodal ghost:
    //   just past the point where a metastable root merges with the unstable branch,
    //   |grad Omega| has a minimum of ~1e-6 and no root; FP64 Newton from the same seed stalls
    //   on it for its whole budget (and so does its trust-region fallback), and the candidate
    //   ends unconverged either way.  The seed is abandoned when the Omega of its best state
    //   lies above the bound by more than 1e-4 |bound| (continuing could only change the
    //   selection by reaching a root that far below from a point where |grad Omega| is a few
    //   1e-6), or at once with `give_up` -- a per-point seed whose point the MultiSeed
    //   candidates judge when it fails (the learned seed).  One float-float thermo pass, once.
    //   Its trust-region fallback then skips a result on the same plateau (seed_fallback).
    // * Give-up: with `give_up` the seed is also abandoned when it still stalls after
    //   kGiveUpRefresh float-float Jacobians (a slowly converging, nearly singular root): the
    //   learned seed is a stand-in for the MultiSeed initial guess, and where it is slow the
    //   MultiSeed candidates decide, as the reference does (no trust-region run of the learned
    //   seed itself).
    // *th_out on these exits: -2 the per-point seed gave up, -3 a plateau above the bound.
    // Without a per-point root, the plateau test takes seed 0's certified Omega as its bound
    // (`anc`, see Anchor).  (Using it in the Omega prune as well made no difference to the
    // bench steps and added waits in MultiSeed table mode.)
    static constexpr int kMaxRefreshJ = 12;
    static constexpr int kGiveUpRefresh = 3;
    static constexpr int kPlateauSteps = 2;
    static constexpr double kPlateauFtol = 1e3;
    static constexpr double kPruneNear = 1e-5, kPruneFFRtol = 1e-9, kPruneFFSlack = 20.0;

    // The rescue of a mixed-precision seed whose refinement stopped contracting, or whose
    // refined state the FP64 residual did not certify.  Such roots are nearly singular:
    // Newton converges on them, but linearly.  With ff_first (a stalled refinement) Newton
    // steps run first on the float-float pass alone -- residual and Jacobian at once, ~1e-12
    // accurate, on the FP32 pipe -- until its residual is below ftol/10 (or stops falling
    // below ftol), as in the refinement; then Newton steps x <- x - J^-1 F with F the FP64
    // residual of the certification pass and J the float-float Jacobian, under NLsolve's stop
    // rules (||F||_inf < ftol, ||dx||_inf < xtol, non-finite values, the budget): at a root
    // the first FP64 residual certifies it.  The outputs come from the float-float thermo
    // pass.  A float-float step costs a single warp about a quarter of a certification pass
    // and a tenth of an FP64 Hessian pass: a rescue is often the last work of a launch.
    // Without the float-float tables it is the FP64 Newton iteration.
    __device__ __noinline__ void newton_rescue(const PointIn &pt, const double *x0, const SolveOpts &o,
                                               Candidate &c, int max_iter, bool ff_first) {
        double x[5], xold[5], p[5], F[5], Fj[5], J[25];
        for (int i = 0; i < 5; ++i) { x[i] = x0[i]; xold[i] = qnan(); }
        if (!eval_newton_ff(pt, x, Fj, J)) {
            newton(pt, x0, o, c, max_iter);
            return;
        }
        int it = 0;
        if (ff_first) {
            double fprev = 1e300;
            while (it < max_iter) {
                const double fn = norm_inf5(Fj);
                if (!(fn == fn) || any_nan5(x)) break;
                if (fn < 0.1 * o.ftol || (fn < o.ftol && !(fn < 0.5 * fprev))) break;
                if (lu_solve5(J, Fj, p)) {
                    for (int i = 0; i < 5; ++i) p[i] = -p[i];
                } else {
                    levenberg_step(J, Fj, p);
                }
                symmetrize_step(pt, x, p);
                double dx = 0.0;
                for (int i = 0; i < 5; ++i) {
                    x[i] += p[i];
                    dx = fabs(p[i]) > dx ? fabs(p[i]) : dx;
                }
                ++it;
                fprev = fn;
                if (!eval_newton_ff(pt, x, Fj, J)) {  // float-float not finite here: an FP64 Jacobian
                    double Fd[5];
                    eval_newton(pt, x, Fd, J);
                    break;
                }
                if (!(dx >= o.xtol)) break;
            }
            if (any_nan5(x)) {  // back to the best state known; the FP64 steps take over
                for (int i = 0; i < 5; ++i) x[i] = x0[i];
                if (!eval_newton_ff(pt, x, Fj, J)) {
                    newton(pt, x0, o, c, max(max_iter - it, 1));
                    c.iterations += it;
                    return;
                }
            }
        }
        eval_grad64(pt, x, F);
        c.exception = !all_finite5(F);
        if (c.exception) {
            for (int i = 0; i < 5; ++i) c.x[i] = x0[i];
            c.residual_norm = qnan();
            c.iterations = it;
            c.f_converged = false;
            c.phys = false;
            return;
        }
        bool xconv = false, fconv = norm_inf5(F) < o.ftol;
        bool stopped = any_nan5(x) || any_nan5(F);
        bool converged = fconv;
        while (!stopped && !converged && it < max_iter) {
            ++it;
            if (lu_solve5(J, F, p)) {
                for (int i = 0; i < 5; ++i) p[i] = -p[i];
            } else {
                levenberg_step(J, F, p);
            }
            symmetrize_step(pt, x, p);
            for (int i = 0; i < 5; ++i) { xold[i] = x[i]; x[i] += p[i]; }
            eval_grad64(pt, x, F);
            double dx = 0.0;
            bool dxn = false;
            for (int i = 0; i < 5; ++i) {
                const double d = fabs(x[i] - xold[i]);
                dxn |= isnan(d);
                dx = d > dx ? d : dx;
            }
            xconv = !any_nan5(xold) && !dxn && dx < o.xtol;
            fconv = norm_inf5(F) < o.ftol;
            stopped = any_nan5(x) || any_nan5(F);
            converged = xconv || fconv;
            if (!stopped && !converged && it < max_iter && !eval_newton_ff(pt, x, Fj, J)) {
                double Fd[5];
                eval_newton(pt, x, Fd, J);  // float-float not finite here: an FP64 Jacobian
            }
        }
        for (int i = 0; i < 5; ++i) c.x[i] = x[i];
        c.residual_norm = norm_inf5(F);
        c.iterations = it;
        c.f_converged = fconv;
        if (!eval_thermo_ff(pt, o, c)) eval_thermo(pt, o, c);
    }

    __device__ bool refine64(const PointIn &pt, const SolveOpts &o, const double *J32, const double *x32, Candidate &c,
                             int &steps, int budget, int *th_out, double bound, bool give_up,
                             const Anchor *anc = nullptr) {
        double F[5], Fo[5], p[5], B[25], xb[5], Jn[25];
        double plast = 0.0;    // |p|inf of the last step
        bool fresh = false;    // the last step used a float-float Jacobian computed at its start
        int plateau = 0;       // consecutive such steps that did not halve the residual
        bool judged = !give_up && !(bound == bound) && !anc;  // the plateau test has run (or cannot)
        for (int i = 0; i < 25; ++i) B[i] = J32[i];
        for (int i = 0; i < 5; ++i) c.x[i] = xb[i] = x32[i];
        c.exception = false;
        c.phys = false;
        c.omega = c.entropy = qnan();
        bool use_ff = eval_grad_ff(pt, c.x, F);
        if (!use_ff) eval_grad64(pt, c.x, F);
        bool is64 = !use_ff;  // F is an FP64 residual
        bool th_valid = false;  // c's thermo fields are those of the current c.x
        steps = 0;
        int refresh = 0;
        if (budget < 2) budget = 2;  // at least one correction and its certification
        double fb = 1e300, fprev = 1e300;
        for (;;) {
            const double fn = norm_inf5(F);
            c.residual_norm = fn;
            const bool bad = !(fn == fn) || any_nan5(c.x);
            if (bad && !is64) {  // float-float residual not usable here: FP64 from now on
                use_ff = false;
                eval_grad64(pt, c.x, F);
                is64 = true;
                continue;
            }
            if (!bad && is64 && fn < o.ftol) { c.f_converged = true; break; }
            if (!bad && fn < fb) {
                for (int i = 0; i < 5; ++i) xb[i] = c.x[i];
                fb = fn;
            }
            if (!bad && !is64 && th_valid && bound == bound && steps > 0 && fn < kPruneNear && fn < 0.5 * fprev &&
                c.omega > bound + kPruneFFRtol * fmax(fabs(bound), 1.0) + kPruneFFSlack * fn * fmax(plast, 1e-3)) {
                cnt.v[kStatPruned] += 1;  // the Omega prune (see above)
                c.f_converged = false;
                *th_out = -1;  // converging to a root that cannot win: no fallback either
                return false;
            }
            if (!bad && !is64 && (fn < 0.1 * o.ftol || (fn < o.ftol && !(fn < 0.5 * fprev)))) {
                *th_out = th_valid ? 1 : 0;  // certification attempt at the current state
                return true;
            }
            const bool stalled = steps > 0 && !(fn < 0.5 * fprev);
            if (steps >= budget) {  // the seed's iteration budget is spent: not converged
                c.f_converged = false;
                if (!is64) { eval_grad64(pt, c.x, F); c.residual_norm = norm_inf5(F); }
                break;
            }
            if (stalled && fresh) ++plateau;
            else if (!stalled) plateau = 0;
            const bool slow = give_up && stalled && refresh >= kGiveUpRefresh;
            if (!judged && ((plateau >= kPlateauSteps && fb > kPlateauFtol * o.ftol) || slow)) {
                judged = true;  // the plateau test (see above), at the best state
                const double pb = (bound == bound || !anc) ? bound : anchor_bound(*anc);
                double xc[5];
                for (int i = 0; i < 5; ++i) { xc[i] = c.x[i]; c.x[i] = xb[i]; }
                if ((give_up || pb == pb) && eval_thermo_ff(pt, o, c) &&
                    (give_up || c.omega > pb + kPruneTightRtol * fmax(fabs(pb), 1.0))) {
                    cnt.v[kStatPruned] += 1;
                    c.f_converged = false;
                    c.residual_norm = fb;
                    *th_out = give_up ? -2 : -3;
                    return false;
                }
                for (int i = 0; i < 5; ++i) c.x[i] = xc[i];
                th_valid = false;
            }
            if (bad || (stalled && refresh >= kMaxRefreshJ)) {
                const int used = steps;
                cnt.v[kStatRescue64] += 1;
                newton_rescue(pt, xb, o, c, budget - used, true);
                steps = used + c.iterations;
                return false;
            }
            fresh = false;
            if (stalled) {
                // a Newton step with the float-float Jacobian at x (its residual replaces F:
                // same accuracy); without float-float, a fresh FP32 Jacobian
                double Fn[5];
                if (use_ff && eval_newton_ff(pt, c.x, Fn, Jn)) {
                    for (int i = 0; i < 5; ++i) F[i] = Fn[i];
                    fresh = true;
                } else {
                    eval_newton32(pt, c.x, Fn, Jn);
                }
                for (int i = 0; i < 25; ++i) B[i] = Jn[i];
                ++refresh;
            }
            fprev = fn;
            if (lu_solve5<true>(B, F, p)) {
                for (int i = 0; i < 5; ++i) p[i] = -p[i];
            } else {
                levenberg_step(B, F, p);
            }
            symmetrize_step(pt, c.x, p);
            plast = 0.0;
            for (int i = 0; i < 5; ++i) {
                c.x[i] += p[i];
                Fo[i] = F[i];
                plast = fabs(p[i]) > plast ? fabs(p[i]) : plast;
            }
            ++steps;
            // after a correction step the state is usually final: the float-float pass also
            // returns the outputs at it
            const int ffr = use_ff ? eval_grad_thermo_ff(pt, o, c, F) : 0;
            th_valid = (ffr & 2) != 0;
            if (ffr & 1) {
                is64 = false;
            } else {
                use_ff = false;
                eval_grad64(pt, c.x, F);
                is64 = true;
            }
            double pp = 0.0;
            for (int i = 0; i < 5; ++i) pp += p[i] * p[i];
            if (pp > 0.0) {
                for (int i = 0; i < 5; ++i) {
                    double r = F[i] - Fo[i];
                    for (int j = 0; j < 5; ++j) r -= B[i * 5 + j] * p[j];
                    r /= pp;
                    for (int j = 0; j < 5; ++j) B[i * 5 + j] += r * p[j];
                }
            }
        }
        // the outputs at the final state: from its float-float residual pass when that was
        // the last one, else a float-float thermo pass (FP64 pass if unavailable)
        if (!th_valid && !eval_thermo_ff(pt, o, c)) eval_thermo(pt, o, c);
        return false;
    }

    // Mixed-precision counterpart of solve_seed.  `dup` is set when the FP32 solution is a
    // root that the dedup policy `dd` has already seen (the same FP64 root, which this seed
    // cannot take from an earlier one under the min-Omega tie rule); then no FP64 work is
    // spent on it.  D provides seen(x) and remember(x), uniform over the group.
    // With `cs` (fused kernel with certifying warps) a seed whose refinement reaches its FP64
    // certification returns true at that point with `out` and `cs` holding its state: the
    // certifying warp finishes it (mixed_seed_finish).  Otherwise the seed is finished here,
    // by the same steps.
    template <class D>
    __device__ __noinline__ bool mixed_solve_seed(const PointIn &pt, const double *x0, const SolveOpts &o, Candidate &out,
                                                  bool &converged, bool &dup, D &dd, CertState *cs = nullptr) {
        cnt.v[kStatSeeds] += 1;
        dup = false;
        out.unstable = false;
        double x32[5], J32[25];
        int it32 = 0;
        const int r = newton32(pt, x0, o, x32, J32, it32, dd.prior_root());
        if (r < 0) {  // decide a non-finite FP32 residual at the seed with the FP64 path
            cnt.v[kStatSeeds] -= 1;
            solve_seed(pt, x0, o, out, converged);
            return false;
        }
        out.exception = false;
        if (r > 0) {
            if (dd.seen(x32)) { dup = true; converged = false; return false; }
            dd.remember(x32);
            if (cannot_win(pt, x32, dd.omega_bound())) { dup = true; converged = false; return false; }
            if (!cs) dd.pending(x32);
            CertState s;
            s.steps = 0;
            s.th_valid = 0;
            // only where the result may be verified; J32 before the refinement's Broyden updates
            s.unstable = o.verify_seeds > 0 && dd.per_point() && det5_negative(J32) ? 1 : 0;
            Anchor an;
            const bool has_an = dd.plateau_anchor(an);
            if (refine64(pt, o, J32, x32, out, s.steps, o.max_iter - it32, &s.th_valid, dd.omega_bound(),
                         o.verify_seeds > 0 && dd.per_point(), has_an ? &an : nullptr)) {
                for (int k = 0; k < 5; ++k) s.x32[k] = x32[k];
                s.it32 = it32;
                if (cs) {
                    *cs = s;
                    return true;
                }
                mixed_seed_finish(pt, x0, o, out, converged, dd, s);
                return false;
            }
            out.iterations = it32 + s.steps;
            dd.withdraw();
            if (s.th_valid == -1) { dup = true; converged = false; return false; }  // cannot win
            if (s.th_valid == -2) { converged = false; return false; }  // the MultiSeed candidates decide
            if (s.th_valid == -3) {  // a plateau above the bound: skip a fallback root on it
                double xp[5];
                for (int k = 0; k < 5; ++k) xp[k] = out.x[k];
                seed_fallback(pt, x0, o, out, converged, dd, xp);
                return false;
            }
        } else {
            for (int i = 0; i < 5; ++i) out.x[i] = x32[i];
            out.f_converged = false;
            out.phys = false;
            out.residual_norm = out.omega = out.entropy = qnan();
            for (int k = 0; k < 3; ++k) out.rho[k] = out.nq[k] = out.naq[k] = qnan();
            out.iterations = it32;
        }
        seed_fallback(pt, x0, o, out, converged, dd);
        return false;
    }

    // FP64 certification of the refined state c.x (refine64 returned true): the root is
    // accepted when the FP64 residual ||grad_x Omega||_inf < ftol.  A state it does not
    // certify (float-float and FP64 disagree, rare) is finished by newton_rescue for the rest
    // of the seed's budget.  `steps` counts the refinement steps on entry and on exit.
    __device__ void certify(const PointIn &pt, const SolveOpts &o, Candidate &c, int &steps, int budget, int th_valid) {
        double F[5];
        eval_grad64(pt, c.x, F);
        const double fn = norm_inf5(F);
        if (fn < o.ftol) {
            c.residual_norm = fn;
            c.f_converged = true;
            if (!th_valid && !eval_thermo_ff(pt, o, c)) eval_thermo(pt, o, c);
            return;
        }
        double xs[5];
        for (int k = 0; k < 5; ++k) xs[k] = c.x[k];
        cnt.v[kStatRescue64] += 1;
        if (budget < 2) budget = 2;
        newton_rescue(pt, xs, o, c, max(budget - steps, 1), false);
        steps += c.iterations;
    }

    // The certification of a deferred seed (see mixed_solve_seed) and the rest of its solve.
    template <class D>
    __device__ __noinline__ void mixed_seed_finish(const PointIn &pt, const double *x0, const SolveOpts &o,
                                                   Candidate &out, bool &converged, D &dd, const CertState &cs) {
        int st = cs.steps;
        certify(pt, o, out, st, o.max_iter - cs.it32, cs.th_valid);
        out.iterations = cs.it32 + st;
        out.unstable = cs.unstable != 0;
        if (cand_good(out, o.residual_norm_max)) dd.publish(cs.x32);
        else dd.withdraw();
        seed_fallback(pt, x0, o, out, converged, dd);
    }

    // The reference's trust-region fallback for an unusable Newton result
    // (ImplicitSolver.jl:130-151, FP32 passes here) and the seed's final verdict.
    // With `plateau` (the state where the Newton result was abandoned on a plateau above the
    // bound), a trust-region result within 1e-3 of it is on the same plateau and is not
    // refined: its Omega is as far above the bound.
    template <class D>
    __device__ void seed_fallback(const PointIn &pt, const double *x0, const SolveOpts &o, Candidate &out,
                                  bool &converged, D &dd, const double *plateau = nullptr) {
        if (!cand_good(out, o.residual_norm_max) && o.trust_region_fallback) {
            cnt.v[kStatTrRuns] += 1;
            double y32[5], K32[25];
            int itt = 0;
            if (tr32(pt, x0, o, y32, K32, itt) > 0 && !dd.seen(y32)) {
                dd.remember(y32);
                bool same = plateau != nullptr;
                for (int k = 0; k < 5 && same; ++k) same = fabs(y32[k] - plateau[k]) <= 1e-3 * (1.0 + fabs(plateau[k]));
                if (same || cannot_win(pt, y32, dd.omega_bound())) {  // the Newton result stays, unusable
                    if (same) cnt.v[kStatPruned] += 1;
                    converged = false;
                    return;
                }
                Candidate f;
                const bool unst = o.verify_seeds > 0 && dd.per_point() && det5_negative(K32);
                int st = 0, th = 0;
                // (no seed-0 bound here: this also runs on certifying warps, which must not wait
                // for a seed whose certification may be queued for them)
                if (refine64(pt, o, K32, y32, f, st, o.max_iter - itt, &th, dd.omega_bound(), o.verify_seeds > 0 && dd.per_point()))
                    certify(pt, o, f, st, o.max_iter - itt, th);
                f.iterations = itt + st;
                f.unstable = unst;
                if (cand_good(f, o.residual_norm_max)) dd.publish(y32);
                if (choose_fallback(out, f, o.residual_norm_max)) out = f;
            }
        }
        converged = cand_good(out, o.residual_norm_max);
    }

    // solve(::FixedMu) single-seed path without the MultiSeed fallback (ImplicitSolver.jl:261-304)
    __device__ void solve_seed(const PointIn &pt, const double *x0, const SolveOpts &o, Candidate &out, bool &converged) {
        cnt.v[kStatSeeds] += 1;
        newton(pt, x0, o, out);
        converged = false;
        if (out.exception) return;
        const bool need = o.trust_region_fallback &&
                          (!out.f_converged || !isfinite(out.residual_norm) || out.residual_norm > o.residual_norm_max ||
                           !out.phys);
        if (need) {
            Candidate f;
            trust_region(pt, x0, o, f);
            if (!f.exception && choose_fallback(out, f, o.residual_norm_max)) out = f;
        }
        converged = cand_good(out, o.residual_norm_max);
    }
};

// ---------------------------------------------------------------------------------------
// States of a (slot, seed) root flag: no root; a root being certified; a certified, usable root.
constexpr int kRootNone = 0, kRootPending = 1, kRootUsable = 2;
// A pending root's verdict comes at the end of one seed's certification (FP64 passes and at
// most the rest of its iteration budget): polled with a sleep, and given up after about
// SolveOpts::verdict_polls x kVerdictSleepNs (then the waiting seed certifies the root itself,
// the result it reaches without waiting).
constexpr unsigned kVerdictSleepNs = 128;

__device__ __forceinline__ int wait_verdict(const int *flag, unsigned polls) {
    int f = *(volatile const int *)flag;
    for (unsigned k = 0; f == kRootPending && k < polls; ++k) {
        __nanosleep(kVerdictSleepNs);
        f = *(volatile const int *)flag;
    }
    return f;
}

// Duplicate-root test of two FP32 solutions (both within the FP32 noise of one root).
__device__ __forceinline__ bool same_root(const double *x, const double *y) {
    bool same = true;
    for (int i = 0; i < 5; ++i) same = same && fabs(x[i] - y[i]) <= 1e-6 * (1.0 + fabs(x[i]));
    return same;
}

// Dedup policy of a single seed solved alone: its Newton root against its trust-region root.
struct LocalRoots {
    double r[2 * 5];
    int n = 0;
    __device__ bool seen(const double *x) const {
        for (int k = 0; k < n; ++k)
            if (same_root(x, r + 5 * k)) return true;
        return false;
    }
    __device__ void remember(const double *x) {
        if (n >= 2) return;
        for (int i = 0; i < 5; ++i) r[5 * n + i] = x[i];
        ++n;
    }
    __device__ double omega_bound() const { return __longlong_as_double(0x7ff8000000000000ll); }
    __device__ bool plateau_anchor(Anchor &) const { return false; }
    __device__ const double *prior_root() const { return nullptr; }
    __device__ bool per_point() const { return true; }
    __device__ void publish(const double *) {}
    __device__ void pending(const double *) {}
    __device__ void withdraw() {}
};

// Dedup policy of the task kernel.  Seed s of a slot skips its FP64 work when its FP32 root
// equals that of an earlier seed s' < s of the same slot whose candidate is already certified
// and usable (see publish()), or `prior`, the certified root of the slot's per-point seed in
// verification mode.  Only such earlier seeds suppress a later one, and a suppressed seed
// would reach the same FP64 root and lose the min-Omega tie to the earlier seed.  An earlier
// seed still certifying the same root (pending()) is waited for when wait_pending is set, so
// the later seed ends as it would had the earlier one finished first; with certification
// deferred to certifying warps it is not (both are refined, the tie rule keeps the earlier).
// Waits point only to earlier seeds that are certifying, which wait for nothing before their
// verdict, so every wait ends.  omega_bound() is the per-point candidate's Omega (verification mode)
// -- a bound fixed before any task of the slot starts, so which candidates are discarded as
// unable to win does not depend on timing; in MultiSeed table mode there is none.  (A bound
// from the seeds of the slot certified so far was tried: with it a candidate dropped on a
// plateau in one run could, in a run where that bound came later, leave the plateau and
// reach a root tied with the minimum -- 18 of 3,000 points chose another of the tied seeds
// between launch forms.)  The leader lane reads and writes; answers are broadcast.  With
// roots = null (a per-point seed, which has no slot) it is LocalRoots alone.
struct PublishedRoots {
    double *roots;        // [slots*S*5]
    int *flag;            // [slots*S]
    int64_t base;         // slot*S
    int s;
    const double *prior;  // or null
    unsigned mask;
    int leader, gl;
    double prior_omega;   // Omega of `prior` (NaN when there is none)
    LocalRoots own;
    bool wait_pending = false;  // wait for the verdict on an earlier seed's pending root
    unsigned verdict_polls = kVerdictPollsDefault;  // bound of that wait and of the anchor wait
    const int *anchor_state = nullptr;     // this slot's seed-0 verdict (Anchor), or null
    const double *anchor_omega = nullptr;
    __device__ double omega_bound() const { return prior_omega; }
    // The plateau bound of a slot without a per-point root, for seeds after seed 0.
    __device__ bool plateau_anchor(Anchor &an) const {
        if (!anchor_state || s == 0 || prior_omega == prior_omega) return false;
        an.state = anchor_state;
        an.omega = anchor_omega;
        an.polls = verdict_polls;
        return true;
    }
    __device__ const double *prior_root() const { return prior; }
    // a per-point seed (no slot), whose root may be sent to the verification seeds
    __device__ bool per_point() const { return roots == nullptr; }
    __device__ bool seen(const double *x) const {
        if (own.seen(x)) return true;
        int hit = 0;
        if (gl == 0) {
            if (prior && same_root(x, prior)) hit = 1;
            for (int q = 0; q < s && !hit; ++q) {
                int f = *(volatile const int *)&flag[base + q];
                if (f == kRootNone) continue;
                __threadfence();
                double y[5];
                for (int i = 0; i < 5; ++i) y[i] = __ldcg(&roots[5 * (base + q) + i]);
                if (f == kRootPending) {
                    // seed q is certifying this root: its verdict decides, as it would had q
                    // finished first (skipped when q's root is usable, refined otherwise)
                    if (!wait_pending || !same_root(x, y)) continue;
                    f = wait_verdict(&flag[base + q], verdict_polls);
                    if (f != kRootUsable) continue;
                    __threadfence();
                    for (int i = 0; i < 5; ++i) y[i] = __ldcg(&roots[5 * (base + q) + i]);
                }
                if (same_root(x, y)) hit = 1;
            }
        }
        return __shfl_sync(mask, hit, leader) != 0;
    }
    __device__ void remember(const double *x) { own.remember(x); }
    // The FP32 root x that this seed goes on to certify, visible to later seeds of the slot
    // as pending until publish() or withdraw() gives the verdict.  Only where the later seeds
    // may wait for it (no deferred certification: the certifying seed runs on, never waiting
    // itself before its verdict, so every wait ends).
    __device__ void pending(const double *x) {
        if (!wait_pending || gl != 0 || !roots || *(volatile const int *)&flag[base + s] != kRootNone) return;
        for (int i = 0; i < 5; ++i) __stcg(&roots[5 * (base + s) + i], x[i]);
        __threadfence();
        atomicExch(&flag[base + s], kRootPending);
    }
    // The pending root was not certified usable.
    __device__ void withdraw() {
        if (gl == 0 && roots && *(volatile const int *)&flag[base + s] == kRootPending)
            atomicExch(&flag[base + s], kRootNone);
    }
    // Publish the FP32 root x of a certified, usable candidate (converged and physical, once
    // per seed): it is this seed's final candidate, so whether a later seed reaching the same
    // root is skipped never changes which candidate the min-Omega selection keeps.  (A root
    // published earlier -- before certification, or unphysical -- could suppress the only
    // seed that ends with a usable candidate for it: a timing-dependent outcome.)
    __device__ void publish(const double *x) {
        if (gl == 0 && roots && *(volatile const int *)&flag[base + s] != kRootUsable) {
            for (int i = 0; i < 5; ++i) __stcg(&roots[5 * (base + s) + i], x[i]);
            __threadfence();
            atomicExch(&flag[base + s], kRootUsable);
        }
    }
};

// ---------------------------------------------------------------------------------------
__device__ __forceinline__ bool valid_point(const PointIn &pt) {
    return isfinite(pt.T) && pt.T > 0.0 && isfinite(pt.mu[0]) && isfinite(pt.mu[1]) && isfinite(pt.mu[2]) &&
           isfinite(pt.xi) && pt.xi > -1.0;
}

__device__ __forceinline__ void load_point(const SolveArgs &a, int64_t i, PointIn &pt) {
    pt.T = a.T[i];
    pt.mu[0] = a.mu_u[i];
    pt.mu[1] = a.mu_d[i];
    pt.mu[2] = a.mu_s[i];
    pt.xi = a.xi[i];
}

__device__ __forceinline__ void nan_candidate(Candidate &c, const double *x) {
    for (int k = 0; k < 5; ++k) c.x[k] = x ? x[k] : qnan();
    c.residual_norm = c.omega = c.entropy = qnan();
    for (int k = 0; k < 3; ++k) c.rho[k] = c.nq[k] = c.naq[k] = qnan();
    c.iterations = 0;
    c.f_converged = c.phys = false;
    c.exception = false;
}

__device__ inline void write_point(const DevParams &P, const PointIn &pt, const pnjl_result_soa &o, int64_t i,
                            const Candidate &c, bool converged, int chosen, int status) {
    double M[3];
    masses(P, c.x, M);
    const double pressure = -c.omega;
    const double rho_norm = (c.rho[0] + c.rho[1] + c.rho[2]) / (3.0 * P.rho0);
    const double energy = -pressure + (pt.mu[0] * c.rho[0] + pt.mu[1] * c.rho[1] + pt.mu[2] * c.rho[2]) + pt.T * c.entropy;
    if (o.x) for (int k = 0; k < 5; ++k) o.x[5 * i + k] = c.x[k];
    if (o.omega) o.omega[i] = c.omega;
    if (o.pressure) o.pressure[i] = pressure;
    if (o.rho_norm) o.rho_norm[i] = rho_norm;
    if (o.entropy) o.entropy[i] = c.entropy;
    if (o.energy) o.energy[i] = energy;
    if (o.masses) for (int k = 0; k < 3; ++k) o.masses[3 * i + k] = M[k];
    if (o.rho) for (int k = 0; k < 3; ++k) o.rho[3 * i + k] = c.rho[k];
    if (o.n_q) for (int k = 0; k < 3; ++k) o.n_q[3 * i + k] = c.nq[k];
    if (o.n_aq) for (int k = 0; k < 3; ++k) o.n_aq[3 * i + k] = c.naq[k];
    if (o.residual_norm) o.residual_norm[i] = c.residual_norm;
    if (o.iterations) o.iterations[i] = c.iterations;
    if (o.chosen_seed) o.chosen_seed[i] = chosen;
    if (o.status) o.status[i] = status;
    if (o.converged) o.converged[i] = converged ? 1 : 0;
}

// Candidate record in the scratch buffer (one slot per (point, seed) task).
__device__ __forceinline__ void store_record(CandRec *r, const Candidate &c, bool converged) {
    for (int k = 0; k < 5; ++k) r->x[k] = c.x[k];
    r->residual_norm = c.residual_norm;
    r->omega = c.omega;
    r->entropy = c.entropy;
    for (int k = 0; k < 3; ++k) { r->rho[k] = c.rho[k]; r->nq[k] = c.nq[k]; r->naq[k] = c.naq[k]; }
    r->iterations = c.iterations;
    r->flags = (c.f_converged ? 1 : 0) | (c.phys ? 2 : 0) | (c.exception ? 4 : 0) | (converged ? 8 : 0);
}

__device__ __forceinline__ void load_record(const CandRec *r, Candidate &c, bool &converged) {
    for (int k = 0; k < 5; ++k) c.x[k] = __ldcg(&r->x[k]);
    c.residual_norm = __ldcg(&r->residual_norm);
    c.omega = __ldcg(&r->omega);
    c.entropy = __ldcg(&r->entropy);
    for (int k = 0; k < 3; ++k) { c.rho[k] = __ldcg(&r->rho[k]); c.nq[k] = __ldcg(&r->nq[k]); c.naq[k] = __ldcg(&r->naq[k]); }
    c.iterations = __ldcg(&r->iterations);
    const int fl = __ldcg(&r->flags);
    c.f_converged = fl & 1;
    c.phys = (fl & 2) != 0;
    c.exception = (fl & 4) != 0;
    converged = (fl & 8) != 0;
}

__device__ __forceinline__ const double *table_row(const SolveArgs &a, const PointIn &pt, int s) {
    const bool hot = pt.T * a.P.hbarc >= a.hot_T_MeV;
    return (hot && a.seed_table_hot) ? a.seed_table_hot + 5 * s : a.seed_table + 5 * s;
}

// The part of needs_verification known before the solve: the point lies in a flagged cell of
// the verification map (or outside it), or below verify_T_max_MeV without a map.
__device__ __forceinline__ bool verification_region(const SolveOpts &o, const PointIn &pt, double hbarc) {
    if (o.verify_seeds <= 0) return false;
    if (o.vmap) {
        const double v[3] = {pt.T, pt.mu[0], pt.xi};
        int64_t idx = 0;
        for (int k = 0; k < 3; ++k) {
            const double f = (v[k] - o.vlo[k]) / (o.vhi[k] - o.vlo[k]) * o.vn[k];
            if (!(f >= 0.0 && f <= (double)o.vn[k])) return true;
            const int c = min((int)f, o.vn[k] - 1);
            idx = idx * o.vn[k] + c;
        }
        return o.vmap[idx] != 0;
    }
    return pt.T * hbarc < o.verify_T_max_MeV;
}

// Whether a converged per-point solution gets the verification seeds: on an unstable branch
// (det5_negative), in the first-order region (a flagged cell of the verification map, or T
// below verify_T_max_MeV without one) or when the root lies far from the seed.
__device__ __forceinline__ bool needs_verification(const SolveOpts &o, const PointIn &pt, double hbarc,
                                                   const double *x0, const double *x, bool unstable) {
    if (o.verify_seeds <= 0) return false;
    if (unstable) return true;  // an unstable branch is never the min-Omega phase: find the others
    if (verification_region(o, pt, hbarc)) return true;
    if (o.verify_max_step > 0.0) {
        double d = 0.0;
        for (int k = 0; k < 5; ++k) d = fmax(d, fabs(x[k] - x0[k]));
        if (!(d <= o.verify_max_step)) return true;
    }
    return false;
}

// Streaming min-Omega rule over seeds in order: a later converged candidate replaces the
// kept one only when its Omega is lower by more than omega_tie_rtol*|Omega| (rtol = 0 is
// the reference's argmin, first minimum kept, SeedStrategies.jl:236-240).
__device__ __forceinline__ bool better(const Candidate &c, const Candidate &best, bool have, double rtol) {
    return !have || c.omega < best.omega - rtol * fabs(best.omega);
}

// MultiSeed over the table inside one group (used by the per-point fallback).
template <int G>
__device__ bool solve_table_inline(Group<G> &grp, const PointIn &pt, const SolveArgs &a, Candidate &best, int &chosen) {
    bool have = false;
    for (int s = 0; s < a.n_seeds; ++s) {
        const double *row = table_row(a, pt, s);
        double x0[5];
        for (int k = 0; k < 5; ++k) x0[k] = row[k];
        Candidate c;
        bool conv;
        grp.solve_seed(pt, x0, a.opts, c, conv);
        if (c.exception || !conv) continue;
        if (better(c, best, have, a.opts.omega_tie_rtol)) { best = c; chosen = s; have = true; }
    }
    return have;
}

}  // namespace pnjl
