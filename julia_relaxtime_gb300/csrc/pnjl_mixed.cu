// pnjl_mixed.cu -- the mixed-precision solve kernels of libpnjl_cuda (PNJL_PREC_MIXED).
//
// Every seed is solved by Group::mixed_solve_seed:
//   1. Newton with FP32 Kahan-compensated node passes (residual and Jacobian), FP64 5x5 solve
//      and update, until the FP32 residual reaches its floor (Group::newton32);
//   2. if this FP32 solution is a root an earlier seed of the point already produced, the
//      seed is a duplicate of that root and costs nothing more;
//   3. otherwise FP64 refinement steps (FP32 Jacobian with Broyden updates) until the FP64
//      residual ||grad_x Omega||_inf < ftol certifies the root (Group::refine64); Omega,
//      entropy, rho_f and n_f come from an FP64 pass at the certified state;
//   4. the reference's fallback logic (trust region when the result is unusable,
//      ImplicitSolver.jl:130-151, here with FP32 passes).
// A residual that is not finite at a seed in FP32 sends that seed down the FP64 path.
//
// Two kernels share the work so that no point's seeds run one after another on one warp:
//   mixed_points_kernel  per-point seed mode (ContinuitySeed-like or learned seeds): one warp
//                        per point solves its own seed; a converged point outside the
//                        verification region is written at once, the others are appended to
//                        a device list (verification: the solution and the first verify_seeds
//                        MultiSeed candidates compete; fallback: the full MultiSeed solve,
//                        ImplicitSolver.jl:306-327);
//   mixed_tasks_kernel   (slot, seed) tasks over the MultiSeed table: every point in table
//                        mode, the listed points after mixed_points_kernel.  The task that
//                        completes a slot's last seed applies the min-Omega selection
//                        (solve_multi, ImplicitSolver.jl:532-559) and writes the point.
// Both are persistent: warps pop work from device queues.  The task kernel reads the list
// length from device memory, so the pair needs no host round trip (and can be captured).
#include "pnjl_group.cuh"

namespace pnjl {

template <int G>
__global__ void __launch_bounds__(kSolveThreads, 2) mixed_points_kernel(SolveArgs a) {
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
    const int S = a.n_seeds;
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
        double x0[5];
        for (int k = 0; k < 5; ++k) x0[k] = a.point_seeds[5 * i + k];
        Candidate single;
        bool conv, dup;
        LocalRoots own;
        grp.mixed_solve_seed(pt, x0, o, single, conv, dup, own);
        if (single.exception) {
            if (gl == 0) write_point(a.P, pt, a.out, i, single, false, -1, PNJL_POINT_EXCEPTION);
            continue;
        }
        int mode = -1;
        if (conv) {
            if (S > 0 && needs_verification(o, pt, a.P.hbarc, x0, single.x)) mode = kListVerify;
        } else if (o.auto_multiseed_fallback && S > 0) {
            mode = kListFallback;
            cnt.v[kStatMsFallbacks] += 1;
        }
        if (gl != 0) continue;
        if (mode < 0) {
            write_point(a.P, pt, a.out, i, single, conv, -1, conv ? PNJL_POINT_CONVERGED : PNJL_POINT_NOT_CONVERGED);
            continue;
        }
        const long long slot = atomicAdd((unsigned long long *)a.list_count, 1ull);
        a.list[slot] = i;
        a.list_mode[slot] = mode;
        store_record(&a.cand[slot * (S + 1) + S], single, conv);
    }
    if (gl == 0)
        for (int k = 0; k < kStatCount; ++k)
            if (cnt.v[k]) atomicAdd((unsigned long long *)&a.stats[k], (unsigned long long)cnt.v[k]);
}

template <int G>
__global__ void __launch_bounds__(kSolveThreads, 2) mixed_tasks_kernel(SolveArgs a) {
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
    const int64_t n_slots = table_mode ? a.n : *(volatile long long *)a.list_count;
    const int64_t n_tasks = n_slots * S;
    while (true) {
        long long t = 0;
        if (gl == 0) t = atomicAdd((unsigned long long *)a.queue2, 1ull);
        t = __shfl_sync(mask, t, leader);
        if (t >= n_tasks) break;
        const int64_t slot = t / S;
        const int s = (int)(t - slot * S);
        const int64_t i = table_mode ? slot : a.list[slot];
        const int mode = table_mode ? kListFull : a.list_mode[slot];
        const int count = mode == kListVerify ? o.verify_seeds : S;
        if (s >= count) continue;
        PointIn pt;
        load_point(a, i, pt);
        CandRec *rec = a.cand + slot * (S + 1);
        if (!valid_point(pt)) {  // table mode only: listed points are valid
            if (s == 0 && gl == 0) {
                Candidate c;
                nan_candidate(c, nullptr);
                write_point(a.P, pt, a.out, i, c, false, -1, PNJL_POINT_INVALID_INPUT);
            }
            continue;
        }
        const double *row = table_row(a, pt, s);
        double x0[5], prior[5];
        for (int k = 0; k < 5; ++k) x0[k] = row[k];
        double prior_omega = qnan();
        if (mode == kListVerify) {
            for (int k = 0; k < 5; ++k) prior[k] = __ldcg(&rec[S].x[k]);
            prior_omega = __ldcg(&rec[S].omega);
        }
        PublishedRoots dd{a.roots, a.root_flag, slot * S, s, mode == kListVerify ? prior : nullptr, mask, leader, gl,
                          prior_omega};
        Candidate c;
        bool conv, dup;
        grp.mixed_solve_seed(pt, x0, o, c, conv, dup, dd);
        int old = 0;
        if (gl == 0) {
            store_record(&rec[s], c, conv);
            if (dup) rec[s].flags |= 16;
            __threadfence();
            old = atomicAdd(&a.done[slot], 1);
        }
        old = __shfl_sync(mask, old, leader);
        if (old != count - 1) continue;
        // this task completed the slot: select among its records
        __threadfence();
        if (gl != 0) continue;
        Candidate best, first;
        bool have = false;
        int chosen = -1, first_idx = -1;
        if (mode == kListVerify) {
            bool cv;
            load_record(&rec[S], best, cv);
            have = true;
        }
        for (int q = 0; q < count; ++q) {
            Candidate cq;
            bool cv;
            load_record(&rec[q], cq, cv);
            if (cq.exception || (__ldcg(&rec[q].flags) & 16)) continue;
            if (first_idx < 0) { first = cq; first_idx = q; }
            if (!cv) continue;
            if (better(cq, best, have, o.omega_tie_rtol)) { best = cq; chosen = q; have = true; }
        }
        if (have) write_point(a.P, pt, a.out, i, best, true, chosen, PNJL_POINT_CONVERGED);
        else if (mode == kListFallback) {
            Candidate single;
            bool cv;
            load_record(&rec[S], single, cv);
            write_point(a.P, pt, a.out, i, single, false, -1, PNJL_POINT_NOT_CONVERGED);
        } else if (first_idx >= 0) write_point(a.P, pt, a.out, i, first, false, first_idx, PNJL_POINT_ALL_SEEDS_FAILED);
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

cudaError_t launch_mixed_points(const SolveArgs &a, int grid, size_t smem, cudaStream_t s) {
    mixed_points_kernel<32><<<grid, kSolveThreads, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_mixed_tasks(const SolveArgs &a, int grid, size_t smem, cudaStream_t s) {
    mixed_tasks_kernel<32><<<grid, kSolveThreads, smem, s>>>(a);
    return cudaGetLastError();
}

int solve_mixed_occupancy(bool tasks, size_t smem) {
    int nb = 0;
    const cudaError_t e =
        tasks ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, mixed_tasks_kernel<32>, kSolveThreads, smem)
              : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, mixed_points_kernel<32>, kSolveThreads, smem);
    return e == cudaSuccess ? nb : 0;
}

}  // namespace pnjl
