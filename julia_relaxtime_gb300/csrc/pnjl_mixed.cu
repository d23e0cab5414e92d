// pnjl_mixed.cu -- the mixed-precision solve kernel of libpnjl_cuda (PNJL_PREC_MIXED).
//
// One warp per point; a point's seeds run one after another in that warp:
//   1. Newton with FP32 Kahan-compensated node passes (residual and Jacobian), FP64 5x5 solve
//      and update, until the FP32 residual reaches its floor (Group::newton32);
//   2. if this FP32 solution equals one an earlier seed of the point already produced, the
//      seed is a duplicate of that root and costs nothing more;
//   3. otherwise FP64 refinement steps with the FP32 Jacobian, x <- x - J32^{-1} F64(x), until
//      the FP64 residual ||grad_x Omega||_inf < ftol certifies the root (Group::refine64);
//      Omega, entropy, rho_f and n_f come from an FP64 pass at the certified state;
//   4. the reference's fallback logic (trust region when the result is unusable,
//      ImplicitSolver.jl:130-151, here with FP32 passes) and min-Omega selection over the
//      seeds (solve_multi, :532-559) are applied to the FP64-certified candidates.
// A residual that is not finite at a seed in FP32 sends that seed down the FP64 path.
#include "pnjl_group.cuh"

namespace pnjl {

template <int G>
__global__ void __launch_bounds__(kSolveThreads, 2) solve_kernel_mixed(SolveArgs a) {
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
    double seen[5 * Group<G>::kMaxSeen];
    while (true) {
        long long t = 0;
        if (gl == 0) t = atomicAdd((unsigned long long *)a.queue, 1ull);
        t = __shfl_sync(mask, t, leader);
        if (t >= a.n) break;
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
        int n_seen = 0;
        Candidate single;
        bool single_conv = false, single_done = false;
        if (!table_mode) {
            double x0[5];
            for (int k = 0; k < 5; ++k) x0[k] = a.point_seeds[5 * i + k];
            bool dup;
            grp.mixed_solve_seed(pt, x0, o, single, single_conv, seen, n_seen, dup);
            if (single.exception) {
                if (gl == 0) write_point(a.P, pt, a.out, i, single, false, -1, PNJL_POINT_EXCEPTION);
                continue;
            }
            if (single_conv && needs_verification(o, pt, a.P.hbarc, x0, single.x)) {
                // a table seed may reach a lower-Omega branch
                Candidate best = single;
                int chosen = -1;
                for (int s = 0; s < o.verify_seeds; ++s) {
                    const double *row = table_row(a, pt, s);
                    double xv[5];
                    for (int k = 0; k < 5; ++k) xv[k] = row[k];
                    Candidate c;
                    bool conv, dup;
                    grp.mixed_solve_seed(pt, xv, o, c, conv, seen, n_seen, dup);
                    if (dup || c.exception || !conv) continue;
                    if (better(c, best, true, o.omega_tie_rtol)) { best = c; chosen = s; }
                }
                if (gl == 0) write_point(a.P, pt, a.out, i, best, true, chosen, PNJL_POINT_CONVERGED);
                continue;
            }
            if (single_conv || !o.auto_multiseed_fallback || a.n_seeds == 0) {
                if (gl == 0)
                    write_point(a.P, pt, a.out, i, single, single_conv, -1,
                                single_conv ? PNJL_POINT_CONVERGED : PNJL_POINT_NOT_CONVERGED);
                continue;
            }
            cnt.v[kStatMsFallbacks] += 1;
            single_done = true;
            n_seen = 0;  // the fallback is a fresh MultiSeed solve (ImplicitSolver.jl:306-327)
        }
        Candidate best, first;
        bool have = false;
        int chosen = -1, first_idx = -1;
        for (int s = 0; s < a.n_seeds; ++s) {
            const double *row = table_row(a, pt, s);
            double x0[5];
            for (int k = 0; k < 5; ++k) x0[k] = row[k];
            Candidate c;
            bool conv, dup;
            grp.mixed_solve_seed(pt, x0, o, c, conv, seen, n_seen, dup);
            if (dup || c.exception) continue;
            if (first_idx < 0) { first = c; first_idx = s; }
            if (!conv) continue;
            if (better(c, best, have, o.omega_tie_rtol)) { best = c; chosen = s; have = true; }
        }
        if (gl != 0) continue;
        if (have) write_point(a.P, pt, a.out, i, best, true, chosen, PNJL_POINT_CONVERGED);
        else if (single_done) write_point(a.P, pt, a.out, i, single, false, -1, PNJL_POINT_NOT_CONVERGED);
        else if (first_idx >= 0) write_point(a.P, pt, a.out, i, first, false, first_idx, PNJL_POINT_ALL_SEEDS_FAILED);
        else {
            Candidate cz;
            nan_candidate(cz, table_row(a, pt, 0));
            write_point(a.P, pt, a.out, i, cz, false, -1, PNJL_POINT_ALL_SEEDS_FAILED);
        }
    }
    if (gl == 0)
        for (int k = 0; k < kStatCount; ++k)
            if (cnt.v[k]) atomicAdd((unsigned long long *)&a.stats[k], (unsigned long long)cnt.v[k]);
}

cudaError_t launch_solve_mixed(const SolveArgs &a, int grid, size_t smem, cudaStream_t s) {
    solve_kernel_mixed<32><<<grid, kSolveThreads, smem, s>>>(a);
    return cudaGetLastError();
}

int solve_mixed_occupancy(size_t smem) {
    int nb = 0;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, solve_kernel_mixed<32>, kSolveThreads, smem) ==
                   cudaSuccess
               ? nb
               : 0;
}

}  // namespace pnjl
