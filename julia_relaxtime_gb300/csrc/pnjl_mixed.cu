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
// The work is split so that no point's seeds run one after another on one warp:
//   per-point seed       (ContinuitySeed-like or learned seeds): one warp per point solves its
//                        own seed; a converged point outside the verification region is
//                        written at once, the others are appended to a device list
//                        (verification: the solution and the first verify_seeds MultiSeed
//                        candidates compete; fallback: the full MultiSeed solve,
//                        ImplicitSolver.jl:306-327);
//   (slot, seed) task    one MultiSeed seed of a listed point (or of every point in table
//                        mode).  The task that completes a slot's last seed applies the
//                        min-Omega selection (solve_multi, ImplicitSolver.jl:532-559) and
//                        writes the point.
// Kernels: mixed_fused_kernel runs both kinds in one launch (listed tasks first, so
// verification seeds overlap the remaining points); mixed_points_kernel followed by
// mixed_tasks_kernel runs them as two launches (the chunk pipeline); mixed_tasks_kernel alone
// runs table mode.  All are persistent: warps pop work from device queues, and no launch needs
// a host round trip (so every form can be captured into a graph).
#include "pnjl_group.cuh"

namespace pnjl {

// The per-point seed of point i (one group).  A converged point outside the verification
// region is written at once; the others are appended to the device list: the point index,
// its record (slot S of the slot's candidates) and, last, its mode + 1, which marks the slot
// complete for a task that is already waiting on it.
template <int G>
__device__ void point_step(Group<G> &grp, const SolveArgs &a, int64_t i, int gl, Counters &cnt) {
    const SolveOpts &o = a.opts;
    const int S = a.n_seeds;
    PointIn pt;
    load_point(a, i, pt);
    if (!valid_point(pt)) {
        if (gl == 0) {
            Candidate c;
            nan_candidate(c, nullptr);
            write_point(a.P, pt, a.out, i, c, false, -1, PNJL_POINT_INVALID_INPUT);
        }
        return;
    }
    double x0[5];
    for (int k = 0; k < 5; ++k) x0[k] = a.point_seeds[5 * i + k];
    Candidate single;
    bool conv, dup;
    // no slot: dedup within the seed's own runs only (the same instantiation of the solve
    // as the tasks', so that the fused kernel holds one copy of it)
    PublishedRoots own{nullptr, nullptr, 0, 0, nullptr, grp.mask, grp.leader(), gl, qnan()};
    grp.mixed_solve_seed(pt, x0, o, single, conv, dup, own);
    if (single.exception) {
        if (gl == 0) write_point(a.P, pt, a.out, i, single, false, -1, PNJL_POINT_EXCEPTION);
        return;
    }
    int mode = -1;
    if (conv) {
        if (S > 0 && needs_verification(o, pt, a.P.hbarc, x0, single.x)) mode = kListVerify;
    } else if (o.auto_multiseed_fallback && S > 0) {
        mode = kListFallback;
        cnt.v[kStatMsFallbacks] += 1;
    }
    if (gl != 0) return;
    if (mode < 0) {
        write_point(a.P, pt, a.out, i, single, conv, -1, conv ? PNJL_POINT_CONVERGED : PNJL_POINT_NOT_CONVERGED);
        return;
    }
    const long long slot = atomicAdd((unsigned long long *)a.list_count, 1ull);
    a.list[slot] = i;
    store_record(&a.cand[slot * (S + 1) + S], single, conv);
    __threadfence();
    atomicExch(&a.list_mode[slot], mode + 1);
}

// Polls of a task on a listed slot whose point is still being written (a few stores by a
// running group; the limit is never reached in practice) and sleep per poll (ns).
constexpr unsigned kReadyPolls = 1u << 24;
constexpr unsigned kReadySleepNs = 64;

// Task t = (slot, seed) of the task list.  The task that completes a slot's last seed applies
// the min-Omega selection and writes the point.
template <int G>
__device__ void task_step(Group<G> &grp, const SolveArgs &a, int64_t t, bool table_mode, int gl, unsigned mask,
                          int leader, Counters &cnt) {
    const SolveOpts &o = a.opts;
    const int S = a.n_seeds;
    const int64_t slot = t / S;
    const int s = (int)(t - slot * S);
    int64_t i;
    int mode;
    if (table_mode) {
        i = slot;
        mode = kListFull;
    } else {
        int m = 0;
        if (gl == 0) {
            m = *(volatile const int *)&a.list_mode[slot];
            for (unsigned k = 0; m == 0 && k < kReadyPolls; ++k) {
                __nanosleep(kReadySleepNs);
                m = *(volatile const int *)&a.list_mode[slot];
            }
        }
        m = __shfl_sync(mask, m, leader);
        if (m == 0) {  // the slot never completed: counted, the host reports it
            cnt.v[kStatWaitTimeouts] += 1;
            return;
        }
        __threadfence();
        i = __ldcg(&a.list[slot]);
        mode = m - 1;
    }
    const int count = mode == kListVerify ? o.verify_seeds : S;
    if (s >= count) return;
    PointIn pt;
    load_point(a, i, pt);
    CandRec *rec = a.cand + slot * (S + 1);
    if (!valid_point(pt)) {  // table mode only: listed points are valid
        if (s == 0 && gl == 0) {
            Candidate c;
            nan_candidate(c, nullptr);
            write_point(a.P, pt, a.out, i, c, false, -1, PNJL_POINT_INVALID_INPUT);
        }
        return;
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
    if (old != count - 1) return;
    // this task completed the slot: select among its records
    __threadfence();
    if (gl != 0) return;
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

template <int G>
__device__ __forceinline__ void flush_counters(const SolveArgs &a, const Counters &cnt, int gl) {
    if (gl == 0)
        for (int k = 0; k < kStatCount; ++k)
            if (cnt.v[k]) atomicAdd((unsigned long long *)&a.stats[k], (unsigned long long)cnt.v[k]);
}

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
    while (true) {
        long long t = 0;
        if (gl == 0) t = atomicAdd((unsigned long long *)a.queue, 1ull);
        t = __shfl_sync(mask, t, leader);
        if (t >= a.n) break;
        point_step(grp, a, t, gl, cnt);
    }
    flush_counters<G>(a, cnt, gl);
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
    const bool table_mode = a.seed_mode == PNJL_SEEDS_TABLE;
    const int S = a.n_seeds;
    const int64_t n_slots = table_mode ? a.n : *(volatile long long *)a.list_count;
    const int64_t n_tasks = n_slots * S;
    while (true) {
        long long t = 0;
        if (gl == 0) t = atomicAdd((unsigned long long *)a.queue2, 1ull);
        t = __shfl_sync(mask, t, leader);
        if (t >= n_tasks) break;
        task_step(grp, a, t, table_mode, gl, mask, leader, cnt);
    }
    flush_counters<G>(a, cnt, gl);
}

// Polls of a group that found no work while points are still being solved (their seeds may
// still defer them), and sleep per poll (ns).  A group that gives up simply exits: the tasks
// listed later are taken by the groups still running, at the latest by the one that listed
// them.
constexpr unsigned kIdlePolls = 1u << 22;
constexpr unsigned kIdleSleepNs = 500;

// Per-point seeds and the tasks they defer in one persistent launch.  A group takes, in this
// order: a listed (slot, seed) task not yet taken; the next point; and, when both queues are
// empty while points are still in flight, waits for their tasks.  Verification seeds thus
// start as soon as their point is listed and share the GPU with the remaining points, instead
// of forming a second launch whose elapsed time is set by its longest seeds.
template <int G>
__global__ void __launch_bounds__(kSolveThreads, 1) mixed_fused_kernel(SolveArgs a) {
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
    const long long S = a.n_seeds;
    unsigned idle = 0;
    while (true) {
        long long t = 0;
        int kind = 0;  // 1 task, 2 point, 0 nothing yet, -1 all work taken
        if (gl == 0) {
            // read "all points finished" before the list length: every slot listed by then
            // is included in it
            const bool all_points = *(volatile const long long *)a.points_done >= a.n;
            __threadfence();
            const long long avail = *(volatile const long long *)a.list_count * S;
            long long h = *(volatile const long long *)a.queue2;
            while (h < avail) {
                const long long old = (long long)atomicCAS((unsigned long long *)a.queue2, (unsigned long long)h,
                                                           (unsigned long long)(h + 1));
                if (old == h) {
                    kind = 1;
                    t = h;
                    break;
                }
                h = old;
            }
            if (kind == 0 && *(volatile const long long *)a.queue < a.n) {
                t = (long long)atomicAdd((unsigned long long *)a.queue, 1ull);
                if (t < a.n) kind = 2;
            }
            if (kind == 0 && all_points) kind = -1;
        }
        kind = __shfl_sync(mask, kind, leader);
        t = __shfl_sync(mask, t, leader);
        if (kind < 0) break;
        if (kind == 0) {
            if (++idle > kIdlePolls) break;
            __nanosleep(kIdleSleepNs);
            continue;
        }
        idle = 0;
        if (kind == 1) {
            task_step(grp, a, t, false, gl, mask, leader, cnt);
        } else {
            point_step(grp, a, t, gl, cnt);
            if (gl == 0) {
                __threadfence();
                atomicAdd((unsigned long long *)a.points_done, 1ull);
            }
        }
    }
    flush_counters<G>(a, cnt, gl);
}

cudaError_t launch_mixed_points(const SolveArgs &a, int grid, size_t smem, cudaStream_t s) {
    mixed_points_kernel<32><<<grid, kSolveThreads, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_mixed_tasks(const SolveArgs &a, int grid, size_t smem, cudaStream_t s) {
    mixed_tasks_kernel<32><<<grid, kSolveThreads, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_mixed_fused(const SolveArgs &a, int grid, size_t smem, cudaStream_t s) {
    mixed_fused_kernel<32><<<grid, kSolveThreads, smem, s>>>(a);
    return cudaGetLastError();
}

int solve_mixed_occupancy(int kernel, size_t smem) {
    int nb = 0;
    cudaError_t e;
    if (kernel == kMixedTasks)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, mixed_tasks_kernel<32>, kSolveThreads, smem);
    else if (kernel == kMixedFused)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, mixed_fused_kernel<32>, kSolveThreads, smem);
    else
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, mixed_points_kernel<32>, kSolveThreads, smem);
    return e == cudaSuccess ? nb : 0;
}

}  // namespace pnjl
