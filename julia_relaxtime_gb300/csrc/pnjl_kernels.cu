// pnjl_kernels.cu -- sm_103a kernels of libpnjl_cuda.
//
//   solve_kernel<G>   persistent: lane groups of G lanes pop tasks from a device work queue.
//                     MultiSeed mode: a task is one (point, seed) pair -- Newton,
//                     trust-region fallback and candidate choice (ImplicitSolver.jl:103-151)
//                     -- whose candidate record goes to a scratch slot; the task that
//                     completes a point's last seed applies the min-Omega selection
//                     (solve_multi, :532-559) and writes the point.  Per-point-seed mode: a
//                     task is one point (single seed, with the MultiSeed fallback inline).
//                     FP64 throughout.
//   eval_kernel<G>    one full pass + assembly per given state (parity checks, thermo).
//
// Host launch wrappers are at the end (called from pnjl_capi.cu).
#include "pnjl_group.cuh"

namespace pnjl {

size_t node_smem_bytes(int p_num, int t_num) {
    // FP64 tables, FP32 tables, float-float low parts, float-float exp tables
    return (size_t)(p_num + t_num) * 2 * (sizeof(double) + 2 * sizeof(float)) + kExpTableFloats * sizeof(float) + 16;
}

template <int G>
__global__ void __launch_bounds__(kSolveThreads, 2) solve_kernel(SolveArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const NodeView nv = stage_nodes(a.nodes, smem_raw);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int gl = lane & (G - 1);
    const unsigned mask = group_mask<G>(lane);
    const int leader = lane & ~(G - 1);
    Counters cnt;
    for (int k = 0; k < kStatCount; ++k) cnt.v[k] = 0;
    Group<G> grp{a.P, nv, gl, mask, cnt};
    const SolveOpts &o = a.opts;
    const bool table_mode = a.seed_mode == PNJL_SEEDS_TABLE;
    const int S = a.n_seeds;
    const int64_t n_tasks = table_mode ? a.n * S : a.n;
    while (true) {
        long long t = 0;
        if (gl == 0) t = atomicAdd((unsigned long long *)a.queue, 1ull);
        t = __shfl_sync(mask, t, leader);
        if (t >= n_tasks) break;
        if (table_mode) {
            const int64_t i = t / S;
            const int s = (int)(t - i * S);
            PointIn pt;
            load_point(a, i, pt);
            if (!valid_point(pt)) {
                if (s == 0 && gl == 0) {
                    Candidate c;
                    nan_candidate(c, nullptr);
                    write_point(a.P, pt, a.out, i, c, false, -1, PNJL_POINT_INVALID_INPUT);
                }
                continue;
            }
            const double *row = table_row(a, pt, s);
            double x0[5];
            for (int k = 0; k < 5; ++k) x0[k] = row[k];
            Candidate c;
            bool conv;
            grp.solve_seed(pt, x0, o, c, conv);
            int old = 0;
            if (gl == 0) {
                store_record(&a.cand[t], c, conv);
                __threadfence();
                old = atomicAdd(&a.done[i], 1);
            }
            old = __shfl_sync(mask, old, leader);
            if (old != S - 1) continue;
            // this task completed the point: select among its S candidate records
            __threadfence();
            if (gl != 0) continue;
            Candidate best, first;
            bool have = false;
            int chosen = -1, first_idx = -1;
            for (int q = 0; q < S; ++q) {
                Candidate cq;
                bool cv;
                load_record(&a.cand[i * S + q], cq, cv);
                if (cq.exception) continue;
                if (first_idx < 0) { first = cq; first_idx = q; }
                if (!cv) continue;
                if (better(cq, best, have, o.omega_tie_rtol)) { best = cq; chosen = q; have = true; }
            }
            if (have) write_point(a.P, pt, a.out, i, best, true, chosen, PNJL_POINT_CONVERGED);
            else if (first_idx >= 0) write_point(a.P, pt, a.out, i, first, false, first_idx, PNJL_POINT_ALL_SEEDS_FAILED);
            else {
                Candidate cz;
                nan_candidate(cz, table_row(a, pt, 0));
                write_point(a.P, pt, a.out, i, cz, false, -1, PNJL_POINT_ALL_SEEDS_FAILED);
            }
        } else {
            const int64_t i = t;
            PointIn pt;
            load_point(a, i, pt);
            if (!valid_point(pt)) {
                if (gl == 0) {
                    Candidate c;
                    nan_candidate(c, nullptr);
                    write_point(a.P, pt, a.out, i, c, false, -1, PNJL_POINT_INVALID_INPUT);
                }
                continue;
            }
            double x0[5];
            for (int k = 0; k < 5; ++k) x0[k] = a.point_seeds[5 * i + k];
            Candidate single;
            bool conv;
            grp.solve_seed(pt, x0, o, single, conv);
            if (single.exception) {
                if (gl == 0) write_point(a.P, pt, a.out, i, single, false, -1, PNJL_POINT_EXCEPTION);
                continue;
            }
            if (conv && o.verify_seeds > 0 &&
                needs_verification(o, pt, a.P.hbarc, x0, single.x, grp.unstable_root(pt, single.x))) {
                Candidate best = single;
                int chosen = -1;
                for (int s = 0; s < o.verify_seeds; ++s) {
                    const double *row = table_row(a, pt, s);
                    double x1[5];
                    for (int k = 0; k < 5; ++k) x1[k] = row[k];
                    Candidate c;
                    bool cv;
                    grp.solve_seed(pt, x1, o, c, cv);
                    if (c.exception || !cv) continue;
                    if (better(c, best, true, o.omega_tie_rtol)) { best = c; chosen = s; }
                }
                if (gl == 0) write_point(a.P, pt, a.out, i, best, true, chosen, PNJL_POINT_CONVERGED);
                continue;
            }
            if (conv || !o.auto_multiseed_fallback || S == 0) {
                if (gl == 0)
                    write_point(a.P, pt, a.out, i, single, conv, -1, conv ? PNJL_POINT_CONVERGED : PNJL_POINT_NOT_CONVERGED);
                continue;
            }
            cnt.v[kStatMsFallbacks] += 1;
            Candidate best;
            int chosen = -1;
            const bool have = solve_table_inline<G>(grp, pt, a, best, chosen);
            if (gl == 0) {
                if (have) write_point(a.P, pt, a.out, i, best, true, chosen, PNJL_POINT_CONVERGED);
                else write_point(a.P, pt, a.out, i, single, false, -1, PNJL_POINT_NOT_CONVERGED);
            }
        }
    }
    if (gl == 0)
        for (int k = 0; k < kStatCount; ++k)
            if (cnt.v[k]) atomicAdd((unsigned long long *)&a.stats[k], (unsigned long long)cnt.v[k]);
}

// One full pass + assembly per state: Omega, grad_x Omega, Hessian_x Omega and thermo
// (MODE 0 FP64, 1 FP32-Kahan); MODE 2: the float-float residual and Jacobian pass alone;
// MODE 3: the FP64 certification residual pass (node_pass_cert) alone; MODE 4: the FP32 Newton
// pass (node_pass_newton32: residual and Jacobian).
template <int G, int MODE>
__global__ void __launch_bounds__(kSolveThreads) eval_kernel(EvalArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const NodeView nv = stage_nodes(a.nodes, smem_raw);
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
        Eval ev;
        double V, V1[3], V2[3];
        if constexpr (MODE >= 2) {
            if constexpr (MODE == 2) {
                node_pass_ff<G, true, false, true>(nv, pt, x, M, gl, mask, S, evals);
            } else if constexpr (MODE == 3) {
                node_pass_cert<G>(nv, pt, x, M, gl, mask, S, evals);
            } else {
                node_pass_newton32<G>(nv, pt, x, M, gl, mask, S, evals);
            }
            vacuum_terms<G>(a.P, M, gl, mask, lane & ~(G - 1), V, V1, V2);
            assemble<true, MODE != 3, false>(a.P, pt, x, M, S, V, V1, V2, ev);
            if (gl == 0) {
                if (a.omega) a.omega[i] = qnan();
                if (a.grad) for (int k = 0; k < 5; ++k) a.grad[5 * i + k] = -ev.F[k];
                if (a.hess) for (int k = 0; k < 25; ++k) a.hess[25 * i + k] = MODE != 3 ? -ev.J[k] : qnan();
            }
            continue;
        } else if constexpr (MODE == 1) {
            node_pass<float, true, true, true, true, G>(nv, pt, x, M, gl, mask, S, evals);
        } else {
            node_pass<double, false, true, true, true, G>(nv, pt, x, M, gl, mask, S, evals);
        }
        vacuum_terms<G>(a.P, M, gl, mask, lane & ~(G - 1), V, V1, V2);
        assemble<true, true, true>(a.P, pt, x, M, S, V, V1, V2, ev);
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
template <int G>
static cudaError_t launch_solve_g(const SolveArgs &a, int grid, size_t smem, cudaStream_t s) {
    solve_kernel<G><<<grid, kSolveThreads, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_solve(const SolveArgs &a, int group, int grid, size_t smem, cudaStream_t s) {
    switch (group) {
        case 32: return launch_solve_g<32>(a, grid, smem, s);
        default: return cudaErrorInvalidValue;
    }
}

template <int G, int MODE>
static cudaError_t launch_eval_g(const EvalArgs &a, int grid, size_t smem, cudaStream_t s) {
    eval_kernel<G, MODE><<<grid, kSolveThreads, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_eval(const EvalArgs &a, int mode, int grid, size_t smem, cudaStream_t s) {
    switch (mode) {
        case 0: return launch_eval_g<32, 0>(a, grid, smem, s);
        case 1: return launch_eval_g<32, 1>(a, grid, smem, s);
        case 2: return launch_eval_g<32, 2>(a, grid, smem, s);
        case 3: return launch_eval_g<32, 3>(a, grid, smem, s);
        case 4: return launch_eval_g<32, 4>(a, grid, smem, s);
        default: return cudaErrorInvalidValue;
    }
}

int solve_kernel_occupancy(int group, size_t smem) {
    int nb = 0;
    cudaError_t e = cudaSuccess;
    switch (group) {
        case 32: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, solve_kernel<32>, kSolveThreads, smem); break;
        default: return 0;
    }
    return e == cudaSuccess ? nb : 0;
}

}  // namespace pnjl
