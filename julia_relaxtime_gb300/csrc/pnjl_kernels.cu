// pnjl_kernels.cu -- sm_103a kernels of libpnjl_cuda.
//
//   solve_kernel<G>   persistent: lane groups of G lanes pop points from a device work
//                     queue (one atomic per point) and run every seed of the point --
//                     Newton, trust-region fallback, candidate choice and min-Omega
//                     selection -- entirely in registers; FP64 throughout.
//   eval_kernel<G>    one pass + assembly per given state (parity checks, thermo).
//
// Host launch wrappers are at the end (called from pnjl_capi.cu).
#include "pnjl_kernels.h"
#include "pnjl_solver.cuh"

namespace pnjl {

// ---------------------------------------------------------------------------------------
// Stage the node tables into shared memory when they fit, else read them from global.
__device__ __forceinline__ NodeView stage_nodes(const KernelNodes &kn, bool fp32_too, void *smem, bool use_smem) {
    NodeView nv;
    nv.n = kn.n;
    if (!use_smem) {
        nv.p2 = kn.p2; nv.pc2 = kn.pc2; nv.w = kn.w;
        nv.p2f = kn.p2f; nv.pc2f = kn.pc2f; nv.wf = kn.wf;
        return nv;
    }
    double *sd = (double *)smem;
    for (int i = threadIdx.x; i < kn.n; i += blockDim.x) {
        sd[i] = kn.p2[i];
        sd[kn.n + i] = kn.pc2[i];
        sd[2 * kn.n + i] = kn.w[i];
    }
    nv.p2 = sd; nv.pc2 = sd + kn.n; nv.w = sd + 2 * kn.n;
    if (fp32_too) {
        float *sf = (float *)(sd + 3 * kn.n);
        for (int i = threadIdx.x; i < kn.n; i += blockDim.x) {
            sf[i] = kn.p2f[i];
            sf[kn.n + i] = kn.pc2f[i];
            sf[2 * kn.n + i] = kn.wf[i];
        }
        nv.p2f = sf; nv.pc2f = sf + kn.n; nv.wf = sf + 2 * kn.n;
    } else {
        nv.p2f = kn.p2f; nv.pc2f = kn.pc2f; nv.wf = kn.wf;
    }
    return nv;
}

struct Counters {
    int64_t passes64, evals64, seeds, tr_runs, ms_fallbacks;
};

template <int G>
struct Group {
    const DevParams &P;
    const NodeView &nv;
    int gl;
    unsigned mask;
    Counters &cnt;

    __device__ void eval_full(const PointIn &pt, const double *x, Eval &ev) {
        double M[3];
        masses(P, x, M);
        PassSums S;
        node_pass<double, false, true, true, G>(nv, pt, x, M, gl, mask, S, cnt.evals64);
        assemble<true, true>(P, pt, x, M, S, ev);
        cnt.passes64 += 1;
    }

    // NLsolve :newton (static line search) from x0
    __device__ void newton(const PointIn &pt, const double *x0, const SolveOpts &o, Candidate &c) {
        Eval ev;
        double x[5], xold[5], p[5];
#pragma unroll
        for (int i = 0; i < 5; ++i) { x[i] = x0[i]; xold[i] = __longlong_as_double(0x7ff8000000000000ll); }
        eval_full(pt, x, ev);
        c.exception = !all_finite5(ev.F);
        if (c.exception) {
            for (int i = 0; i < 5; ++i) c.x[i] = x0[i];
            c.residual_norm = __longlong_as_double(0x7ff8000000000000ll);
            c.iterations = 0;
            c.f_converged = false;
            c.phys = false;
            return;
        }
        int it = 0;
        bool xconv = false, fconv = norm_inf5(ev.F) < o.ftol;
        bool stopped = any_nan5(x) || any_nan5(ev.F);
        bool converged = fconv;
        while (!stopped && !converged && it < o.max_iter) {
            ++it;
            if (lu_solve5(ev.J, ev.F, p)) {
#pragma unroll
                for (int i = 0; i < 5; ++i) p[i] = -p[i];
            } else {
                // singular Jacobian: p = -(J'J + lambda I) \ J'F
                double g[5], A[25], s = 0.0;
                for (int i = 0; i < 5; ++i) {
                    double a = 0.0;
                    for (int k = 0; k < 5; ++k) a += ev.J[k * 5 + i] * ev.F[k];
                    g[i] = a;
                }
                for (int i = 0; i < 5; ++i)
                    for (int j = 0; j < 5; ++j) {
                        double a = 0.0;
                        for (int k = 0; k < 5; ++k) a += ev.J[k * 5 + i] * ev.J[k * 5 + j];
                        A[i * 5 + j] = -a;
                        s += fabs(a);
                    }
                const double lambda = 1e6 * sqrt(5.0 * 2.220446049250313e-16) * s;
                for (int i = 0; i < 5; ++i) A[i * 5 + i] -= lambda;
                if (!lu_solve5(A, g, p))
                    for (int i = 0; i < 5; ++i) p[i] = __longlong_as_double(0x7ff8000000000000ll);
            }
#pragma unroll
            for (int i = 0; i < 5; ++i) { xold[i] = x[i]; x[i] += p[i]; }
            eval_full(pt, x, ev);
            double dx = 0.0;
            bool dxn = false;
#pragma unroll
            for (int i = 0; i < 5; ++i) {
                const double d = fabs(x[i] - xold[i]);
                dxn |= isnan(d);
                dx = d > dx ? d : dx;
            }
            xconv = !any_nan5(xold) && !dxn && dx < o.xtol;
            fconv = norm_inf5(ev.F) < o.ftol;
            stopped = any_nan5(x) || any_nan5(ev.F);
            converged = xconv || fconv;
        }
        for (int i = 0; i < 5; ++i) c.x[i] = x[i];
        c.residual_norm = norm_inf5(ev.F);
        c.iterations = it;
        c.f_converged = fconv;
        postprocess(P, pt, o, ev, c);
    }

    // NLsolve :trust_region (dogleg, autoscale) from x0
    __device__ void trust_region(const PointIn &pt, const double *x0, const SolveOpts &o, Candidate &c) {
        Eval acc, trial;
        double x[5], xold[5], d[5], p[5];
        for (int i = 0; i < 5; ++i) { x[i] = x0[i]; xold[i] = __longlong_as_double(0x7ff8000000000000ll); }
        eval_full(pt, x, acc);
        cnt.tr_runs += 1;
        c.exception = !all_finite5(acc.F);
        if (c.exception) {
            for (int i = 0; i < 5; ++i) c.x[i] = x0[i];
            c.residual_norm = __longlong_as_double(0x7ff8000000000000ll);
            c.iterations = 0; c.f_converged = false; c.phys = false;
            return;
        }
        int it = 0;
        bool xconv = false, fconv = norm_inf5(acc.F) < o.ftol;
        bool stopped = any_nan5(x) || any_nan5(acc.F);
        bool converged = fconv;
        bool last_nan_F = any_nan5(acc.F);
        if (!converged) {
            for (int j = 0; j < 5; ++j) {
                double s = 0.0;
                for (int i = 0; i < 5; ++i) s += acc.J[i * 5 + j] * acc.J[i * 5 + j];
                d[j] = sqrt(s);
                if (d[j] == 0.0) d[j] = 1.0;
            }
            double delta = 0.0;
            for (int i = 0; i < 5; ++i) delta += (d[i] * x[i]) * (d[i] * x[i]);
            delta = sqrt(delta);
            if (delta == 0.0) delta = 1.0;
            while (!stopped && !converged && it < o.max_iter) {
                ++it;
                dogleg(p, acc.F, d, acc.J, delta);
                for (int i = 0; i < 5; ++i) { xold[i] = x[i]; x[i] += p[i]; }
                eval_full(pt, x, trial);
                double sr = 0.0, sf = 0.0, sp = 0.0;
                for (int k = 0; k < 5; ++k) {
                    double a = 0.0;
                    for (int i = 0; i < 5; ++i) a += acc.J[k * 5 + i] * p[i];
                    const double rp = a + acc.F[k];
                    sr += acc.F[k] * acc.F[k];
                    sf += trial.F[k] * trial.F[k];
                    sp += rp * rp;
                }
                const double rho = (sr - sf) / (sr - sp);
                if (rho > 1e-4) {
                    acc = trial;
                    for (int j = 0; j < 5; ++j) {
                        double s = 0.0;
                        for (int i = 0; i < 5; ++i) s += acc.J[i * 5 + j] * acc.J[i * 5 + j];
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
                    xconv = !dxn && dx < o.xtol;
                    fconv = norm_inf5(acc.F) < o.ftol;
                    converged = xconv || fconv;
                } else {
                    for (int i = 0; i < 5; ++i) x[i] -= p[i];
                    xconv = false;
                    converged = false;
                }
                double wp = 0.0;
                for (int i = 0; i < 5; ++i) wp += (d[i] * p[i]) * (d[i] * p[i]);
                wp = sqrt(wp);
                if (rho < 0.1) delta = delta / 2.0;
                else if (rho >= 0.9) delta = 2.0 * wp;
                else if (rho >= 0.5) delta = fmax(delta, 2.0 * wp);
                last_nan_F = any_nan5(trial.F);
                stopped = any_nan5(x) || last_nan_F;
            }
        }
        for (int i = 0; i < 5; ++i) c.x[i] = x[i];
        c.residual_norm = norm_inf5(acc.F);
        c.iterations = it;
        c.f_converged = fconv;
        // acc holds the evaluation at the last accepted x, which is the returned x
        postprocess(P, pt, o, acc, c);
    }

    // Powell dogleg inside ||D p|| <= delta (Nocedal & Wright, algorithm 4.1 family)
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

    // solve(::FixedMu) single-seed path without the MultiSeed fallback (ImplicitSolver.jl:261-304)
    __device__ void solve_seed(const PointIn &pt, const double *x0, const SolveOpts &o, Candidate &out, bool &converged) {
        cnt.seeds += 1;
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
__device__ __forceinline__ bool valid_point(const PointIn &pt) {
    return isfinite(pt.T) && pt.T > 0.0 && isfinite(pt.mu[0]) && isfinite(pt.mu[1]) && isfinite(pt.mu[2]) &&
           isfinite(pt.xi) && pt.xi > -1.0;
}

template <int G>
__device__ void write_point(const DevParams &P, const PointIn &pt, const SolveArgs &a, int64_t i, int gl,
                            const Candidate &c, bool converged, int chosen, int status) {
    if (gl != 0) return;
    double M[3];
    masses(P, c.x, M);
    const double pressure = -c.omega;
    const double rho_norm = (c.rho[0] + c.rho[1] + c.rho[2]) / (3.0 * P.rho0);
    const double energy = -pressure + (pt.mu[0] * c.rho[0] + pt.mu[1] * c.rho[1] + pt.mu[2] * c.rho[2]) + pt.T * c.entropy;
    const pnjl_result_soa &o = a.out;
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

// MultiSeed over the seed table with the streaming tie rule: a later converged candidate
// replaces the kept one only when its Omega is lower by more than omega_tie_rtol*|Omega|
// (rtol = 0 is the reference's argmin with the first minimum kept).
template <int G>
__device__ bool solve_table(Group<G> &grp, const PointIn &pt, const SolveArgs &a, const SolveOpts &o, Candidate &best,
                            int &chosen, Candidate &first, int &first_idx) {
    bool have = false;
    first_idx = -1;
    const bool hot = pt.T * a.P.hbarc >= a.hot_T_MeV;
    for (int s = 0; s < a.n_seeds; ++s) {
        const double *row = (hot && a.seed_table_hot) ? a.seed_table_hot + 5 * s : a.seed_table + 5 * s;
        double x0[5];
        for (int k = 0; k < 5; ++k) x0[k] = row[k];
        Candidate c;
        bool conv;
        grp.solve_seed(pt, x0, o, c, conv);
        if (c.exception) continue;
        if (first_idx < 0) { first = c; first_idx = s; }
        if (!conv) continue;
        if (!have || c.omega < best.omega - o.omega_tie_rtol * fabs(best.omega)) {
            best = c;
            chosen = s;
            have = true;
        }
    }
    return have;
}

template <int G>
__global__ void __launch_bounds__(kSolveThreads) solve_kernel(SolveArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const NodeView nv = stage_nodes(a.nodes, false, smem_raw, a.stage_nodes);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int gl = lane & (G - 1);
    const unsigned mask = group_mask<G>(lane);
    const int leader = lane & ~(G - 1);
    Counters cnt = {0, 0, 0, 0, 0};
    Group<G> grp{a.P, nv, gl, mask, cnt};
    const SolveOpts &o = a.opts;
    while (true) {
        long long idx = 0;
        if (gl == 0) idx = atomicAdd((unsigned long long *)a.queue, 1ull);
        idx = __shfl_sync(mask, idx, leader);
        if (idx >= a.n) break;
        const int64_t i = idx;
        PointIn pt;
        pt.T = a.T[i];
        pt.mu[0] = a.mu_u[i];
        pt.mu[1] = a.mu_d[i];
        pt.mu[2] = a.mu_s[i];
        pt.xi = a.xi[i];
        if (!valid_point(pt)) {
            Candidate c;
            for (int k = 0; k < 5; ++k) c.x[k] = __longlong_as_double(0x7ff8000000000000ll);
            c.residual_norm = c.omega = c.entropy = __longlong_as_double(0x7ff8000000000000ll);
            for (int k = 0; k < 3; ++k) c.rho[k] = c.nq[k] = c.naq[k] = __longlong_as_double(0x7ff8000000000000ll);
            c.iterations = 0;
            write_point<G>(a.P, pt, a, i, gl, c, false, -1, PNJL_POINT_INVALID_INPUT);
            continue;
        }
        Candidate best, first;
        int chosen = -1, first_idx = -1;
        if (a.seed_mode == PNJL_SEEDS_PER_POINT) {
            double x0[5];
            for (int k = 0; k < 5; ++k) x0[k] = a.point_seeds[5 * i + k];
            Candidate single;
            bool conv;
            grp.solve_seed(pt, x0, o, single, conv);
            if (single.exception) {
                write_point<G>(a.P, pt, a, i, gl, single, false, -1, PNJL_POINT_EXCEPTION);
                continue;
            }
            if (conv || !o.auto_multiseed_fallback) {
                write_point<G>(a.P, pt, a, i, gl, single, conv, -1, conv ? PNJL_POINT_CONVERGED : PNJL_POINT_NOT_CONVERGED);
                continue;
            }
            cnt.ms_fallbacks += 1;
            if (solve_table<G>(grp, pt, a, o, best, chosen, first, first_idx))
                write_point<G>(a.P, pt, a, i, gl, best, true, chosen, PNJL_POINT_CONVERGED);
            else
                write_point<G>(a.P, pt, a, i, gl, single, false, -1, PNJL_POINT_NOT_CONVERGED);
        } else {
            if (solve_table<G>(grp, pt, a, o, best, chosen, first, first_idx)) {
                write_point<G>(a.P, pt, a, i, gl, best, true, chosen, PNJL_POINT_CONVERGED);
            } else if (first_idx >= 0) {
                write_point<G>(a.P, pt, a, i, gl, first, false, first_idx, PNJL_POINT_ALL_SEEDS_FAILED);
            } else {
                Candidate c;
                for (int k = 0; k < 5; ++k) c.x[k] = a.seed_table[k];
                c.residual_norm = c.omega = c.entropy = __longlong_as_double(0x7ff8000000000000ll);
                for (int k = 0; k < 3; ++k) c.rho[k] = c.nq[k] = c.naq[k] = __longlong_as_double(0x7ff8000000000000ll);
                c.iterations = 0;
                write_point<G>(a.P, pt, a, i, gl, c, false, -1, PNJL_POINT_ALL_SEEDS_FAILED);
            }
        }
    }
    if (gl == 0) {
        atomicAdd((unsigned long long *)&a.stats[0], (unsigned long long)cnt.passes64);
        atomicAdd((unsigned long long *)&a.stats[1], (unsigned long long)cnt.evals64);
        atomicAdd((unsigned long long *)&a.stats[2], (unsigned long long)cnt.seeds);
        atomicAdd((unsigned long long *)&a.stats[3], (unsigned long long)cnt.tr_runs);
        atomicAdd((unsigned long long *)&a.stats[4], (unsigned long long)cnt.ms_fallbacks);
    }
}

// One pass + assembly per state: Omega, grad_x Omega, Hessian_x Omega and thermo.
template <int G, bool FP32>
__global__ void __launch_bounds__(kSolveThreads) eval_kernel(EvalArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const NodeView nv = stage_nodes(a.nodes, FP32, smem_raw, a.stage_nodes);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int gl = lane & (G - 1);
    const unsigned mask = group_mask<G>(lane);
    const int64_t groups_per_block = blockDim.x / G;
    const int64_t gid = (int64_t)blockIdx.x * groups_per_block + threadIdx.x / G;
    const int64_t stride = (int64_t)gridDim.x * groups_per_block;
    int64_t evals = 0;
    for (int64_t i = gid; i < a.n; i += stride) {
        PointIn pt;
        pt.T = a.T[i];
        pt.mu[0] = a.mu_u[i];
        pt.mu[1] = a.mu_d[i];
        pt.mu[2] = a.mu_s[i];
        pt.xi = a.xi[i];
        double x[5];
        for (int k = 0; k < 5; ++k) x[k] = a.x[5 * i + k];
        double M[3];
        masses(a.P, x, M);
        PassSums S;
        if (FP32) node_pass<float, true, true, true, G>(nv, pt, x, M, gl, mask, S, evals);
        else node_pass<double, false, true, true, G>(nv, pt, x, M, gl, mask, S, evals);
        Eval ev;
        assemble<true, true>(a.P, pt, x, M, S, ev);
        if (gl == 0) {
            if (a.omega) a.omega[i] = ev.omega;
            if (a.grad) for (int k = 0; k < 5; ++k) a.grad[5 * i + k] = -ev.F[k];
            if (a.hess) for (int k = 0; k < 25; ++k) a.hess[25 * i + k] = -ev.J[k];
            const pnjl_result_soa &o = a.out;
            const double pressure = -ev.omega;
            const double entropy = -ev.dOdT;
            const double rho_norm = (ev.rho[0] + ev.rho[1] + ev.rho[2]) / (3.0 * a.P.rho0);
            const double energy =
                -pressure + (pt.mu[0] * ev.rho[0] + pt.mu[1] * ev.rho[1] + pt.mu[2] * ev.rho[2]) + pt.T * entropy;
            if (o.omega) o.omega[i] = ev.omega;
            if (o.pressure) o.pressure[i] = pressure;
            if (o.entropy) o.entropy[i] = entropy;
            if (o.rho_norm) o.rho_norm[i] = rho_norm;
            if (o.energy) o.energy[i] = energy;
            if (o.masses) for (int k = 0; k < 3; ++k) o.masses[3 * i + k] = M[k];
            if (o.rho) for (int k = 0; k < 3; ++k) o.rho[3 * i + k] = ev.rho[k];
            if (o.n_q) for (int k = 0; k < 3; ++k) o.n_q[3 * i + k] = ev.nq[k];
            if (o.n_aq) for (int k = 0; k < 3; ++k) o.n_aq[3 * i + k] = ev.naq[k];
        }
    }
}

// ---------------------------------------------------------------------------------------
// launch wrappers
size_t node_smem_bytes(int n, bool fp32_too) { return (size_t)n * 3 * (sizeof(double) + (fp32_too ? sizeof(float) : 0)); }

template <int G>
static cudaError_t launch_solve_g(const SolveArgs &a, int grid, size_t smem, cudaStream_t s) {
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(solve_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    solve_kernel<G><<<grid, kSolveThreads, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_solve(const SolveArgs &a, int group, int grid, size_t smem, cudaStream_t s) {
    switch (group) {
        case 32: return launch_solve_g<32>(a, grid, smem, s);
        case 8: return launch_solve_g<8>(a, grid, smem, s);
        default: return cudaErrorInvalidValue;
    }
}

template <int G, bool FP32>
static cudaError_t launch_eval_g(const EvalArgs &a, int grid, size_t smem, cudaStream_t s) {
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(eval_kernel<G, FP32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    eval_kernel<G, FP32><<<grid, kSolveThreads, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_eval(const EvalArgs &a, bool fp32, int grid, size_t smem, cudaStream_t s) {
    return fp32 ? launch_eval_g<32, true>(a, grid, smem, s) : launch_eval_g<32, false>(a, grid, smem, s);
}

int solve_kernel_occupancy(int group, size_t smem) {
    int nb = 0;
    cudaError_t e = cudaSuccess;
    switch (group) {
        case 32: cudaFuncSetAttribute(solve_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                 e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, solve_kernel<32>, kSolveThreads, smem); break;
        case 8: cudaFuncSetAttribute(solve_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, solve_kernel<8>, kSolveThreads, smem); break;
        default: return 0;
    }
    return e == cudaSuccess ? nb : 0;
}

}  // namespace pnjl
