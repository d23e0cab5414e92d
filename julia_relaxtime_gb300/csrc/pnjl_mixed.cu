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

// Ready flags of the device lists (list_mode, job_ready) are written last, after a fence, by
// the lane that wrote the entry; a reader that has taken an entry polls its flag (the writer
// is a running group a few stores away from setting it; the default limit, SolveOpts::
// ready_polls, is never reached in practice) and reads the entry through L2.
constexpr unsigned kReadySleepNs = 64;

__device__ __forceinline__ int wait_ready(const int *flag, unsigned polls) {
    int m = *(volatile const int *)flag;
    for (unsigned k = 0; m == 0 && k < polls; ++k) {
        __nanosleep(kReadySleepNs);
        m = *(volatile const int *)flag;
    }
    return m;
}

// Append a deferred seed to the certification queue (lane 0).
__device__ __forceinline__ void push_job(const SolveArgs &a, int kind, long long t, const Candidate &c,
                                         const CertState &cs) {
    const long long j = (long long)atomicAdd((unsigned long long *)a.job_count, 1ull);
    CertJob &jb = a.jobs[j];
    jb.t = t;
    jb.kind = kind;
    jb.flags = (c.f_converged ? 1 : 0) | (c.exception ? 2 : 0) | (c.phys ? 4 : 0);
    jb.iterations = c.iterations;
    jb.cs = cs;
    for (int k = 0; k < 5; ++k) jb.x[k] = c.x[k];
    jb.residual_norm = c.residual_norm;
    jb.omega = c.omega;
    jb.entropy = c.entropy;
    for (int k = 0; k < 3; ++k) { jb.rho[k] = c.rho[k]; jb.nq[k] = c.nq[k]; jb.naq[k] = c.naq[k]; }
    __threadfence();
    atomicExch(&a.job_ready[j], 1);
}

__device__ __forceinline__ void load_job(const CertJob *jp, long long &t, int &kind, Candidate &c, CertState &cs) {
    t = __ldcg(&jp->t);
    kind = __ldcg(&jp->kind);
    const int fl = __ldcg(&jp->flags);
    c.f_converged = fl & 1;
    c.exception = (fl & 2) != 0;
    c.phys = (fl & 4) != 0;
    c.iterations = __ldcg(&jp->iterations);
    for (int k = 0; k < 5; ++k) { cs.x32[k] = __ldcg(&jp->cs.x32[k]); c.x[k] = __ldcg(&jp->x[k]); }
    cs.it32 = __ldcg(&jp->cs.it32);
    cs.steps = __ldcg(&jp->cs.steps);
    cs.th_valid = __ldcg(&jp->cs.th_valid);
    cs.unstable = __ldcg(&jp->cs.unstable);
    c.residual_norm = __ldcg(&jp->residual_norm);
    c.omega = __ldcg(&jp->omega);
    c.entropy = __ldcg(&jp->entropy);
    for (int k = 0; k < 3; ++k) {
        c.rho[k] = __ldcg(&jp->rho[k]);
        c.nq[k] = __ldcg(&jp->nq[k]);
        c.naq[k] = __ldcg(&jp->naq[k]);
    }
}

// The end of point i's own seed: a converged point outside the verification region is
// written at once; the others are appended to the device list -- the point index, its record
// (slot S of the slot's candidates) and, last, its mode + 1, which marks the slot complete
// for a task already waiting on it.  Counts the point as completed (fused kernel).
template <int G>
__device__ void point_complete(const SolveArgs &a, const PointIn &pt, int64_t i, const double *x0,
                               const Candidate &single, bool conv, int gl, Counters &cnt) {
    const SolveOpts &o = a.opts;
    const int S = a.n_seeds;
    int mode = -1;
    if (single.exception) {
        mode = -2;
    } else if (conv) {
        if (S > 0 && needs_verification(o, pt, a.P.hbarc, x0, single.x, single.unstable)) mode = kListVerify;
    } else if (o.auto_multiseed_fallback && S > 0) {
        mode = kListFallback;
        cnt.v[kStatMsFallbacks] += 1;
    }
    if (gl != 0) return;
    if (mode == -2) {
        write_point(a.P, pt, a.out, i, single, false, -1, PNJL_POINT_EXCEPTION);
    } else if (mode < 0) {
        write_point(a.P, pt, a.out, i, single, conv, -1, conv ? PNJL_POINT_CONVERGED : PNJL_POINT_NOT_CONVERGED);
    } else {
        const long long slot = atomicAdd((unsigned long long *)a.list_count, 1ull);
        a.list[slot] = i;
        store_record(&a.cand[slot * (S + 1) + S], single, conv);
        __threadfence();
        atomicExch(&a.list_mode[slot], mode + 1);
    }
    if (a.points_done) {
        __threadfence();
        atomicAdd((unsigned long long *)a.points_done, 1ull);
    }
}

// The per-point seed of point i (one group).  With certifying warps (defer) a seed that
// reaches its FP64 certification is queued instead of completed here.
template <int G>
__device__ void point_step(Group<G> &grp, const SolveArgs &a, int64_t i, int gl, Counters &cnt, bool defer) {
    const SolveOpts &o = a.opts;
    PointIn pt;
    load_point(a, i, pt);
    if (!valid_point(pt)) {
        if (gl == 0) {
            Candidate c;
            nan_candidate(c, nullptr);
            write_point(a.P, pt, a.out, i, c, false, -1, PNJL_POINT_INVALID_INPUT);
            if (a.points_done) {
                __threadfence();
                atomicAdd((unsigned long long *)a.points_done, 1ull);
            }
        }
        return;
    }
    double x0[5];
    for (int k = 0; k < 5; ++k) x0[k] = a.point_seeds[5 * i + k];
    Candidate single;
    bool conv, dup;
    CertState cs;
    // no slot: dedup within the seed's own runs only (the same instantiation of the solve
    // as the tasks', so that the fused kernel holds one copy of it)
    PublishedRoots own{nullptr, nullptr, 0, 0, nullptr, grp.mask, grp.leader(), gl, qnan()};
    if (grp.mixed_solve_seed(pt, x0, o, single, conv, dup, own, defer ? &cs : nullptr)) {
        if (gl == 0) push_job(a, kJobPoint, i, single, cs);
        return;
    }
    point_complete<G>(a, pt, i, x0, single, conv, gl, cnt);
}

// Slot, seed, point and mode of task t (waits for the slot's ready flag in per-point mode).
// False when the slot never became ready (counted; the host reports it).
__device__ __forceinline__ bool task_slot(const SolveArgs &a, int64_t t, bool table_mode, int gl, unsigned mask,
                                          int leader, Counters &cnt, int64_t &slot, int &s, int64_t &i, int &mode) {
    const int S = a.n_seeds;
    slot = t / S;
    s = (int)(t - slot * S);
    if (table_mode) {
        i = slot;
        mode = kListFull;
        return true;
    }
    int m = 0;
    if (gl == 0) m = wait_ready(&a.list_mode[slot], a.opts.ready_polls);
    m = __shfl_sync(mask, m, leader);
    if (m == 0) {
        cnt.v[kStatWaitTimeouts] += 1;
        return false;
    }
    __threadfence();
    i = __ldcg(&a.list[slot]);
    mode = m - 1;
    return true;
}

// The end of a task: its record, and for the task that completes the slot's last seed the
// min-Omega selection over the slot's records and the point's output.
template <int G>
__device__ void task_complete(const SolveArgs &a, const PointIn &pt, int64_t i, int64_t slot, int s, int mode,
                              const Candidate &c, bool conv, bool dup, int gl, unsigned mask, int leader) {
    const SolveOpts &o = a.opts;
    const int S = a.n_seeds;
    const int count = mode == kListVerify ? o.verify_seeds : S;
    CandRec *rec = a.cand + slot * (S + 1);
    int old = 0;
    if (gl == 0) {
        store_record(&rec[s], c, conv);
        if (dup) rec[s].flags |= 16;
        if (s == 0 && a.anchor_state) {  // seed 0's verdict: the slot's plateau bound (Anchor)
            const bool usable = conv && !dup && c.omega == c.omega;
            if (usable) a.anchor_omega[slot] = c.omega;
            __threadfence();
            atomicExch(&a.anchor_state[slot], usable ? 1 : 2);
        }
        __threadfence();
        old = atomicAdd(&a.done[slot], 1);
    }
    old = __shfl_sync(mask, old, leader);
    if (old == count - 1) {
        // this task completed the slot: select among its records
        __threadfence();
        if (gl == 0) {
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
    }
}

// The dedup policy of a task (see PublishedRoots).
__device__ __forceinline__ PublishedRoots task_roots(const SolveArgs &a, int64_t slot, int s, int mode, double *prior,
                                                     unsigned mask, int leader, int gl) {
    const int S = a.n_seeds;
    const CandRec *rec = a.cand + slot * (S + 1);
    double prior_omega = qnan();
    if (mode == kListVerify) {
        for (int k = 0; k < 5; ++k) prior[k] = __ldcg(&rec[S].x[k]);
        prior_omega = __ldcg(&rec[S].omega);
    }
    PublishedRoots dd{a.roots, a.root_flag, slot * S, s, mode == kListVerify ? prior : nullptr, mask, leader, gl,
                      prior_omega};
    if (a.anchor_state) {
        dd.anchor_state = a.anchor_state + slot;
        dd.anchor_omega = a.anchor_omega + slot;
    }
    return dd;
}

// Task t = (slot, seed) of the task list.  With certifying warps (defer) a seed that reaches
// its FP64 certification is queued instead of completed here.
template <int G>
__device__ void task_step(Group<G> &grp, const SolveArgs &a, int64_t t, bool table_mode, int gl, unsigned mask,
                          int leader, Counters &cnt, bool defer = false) {
    const SolveOpts &o = a.opts;
    int64_t slot, i;
    int s, mode;
    if (!task_slot(a, t, table_mode, gl, mask, leader, cnt, slot, s, i, mode)) return;
    const int count = mode == kListVerify ? o.verify_seeds : a.n_seeds;
    if (s >= count) return;
    PointIn pt;
    load_point(a, i, pt);
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
    PublishedRoots dd = task_roots(a, slot, s, mode, prior, mask, leader, gl);
    dd.wait_pending = !defer;
    dd.verdict_polls = a.opts.verdict_polls;
    Candidate c;
    bool conv, dup;
    CertState cs;
    if (grp.mixed_solve_seed(pt, x0, o, c, conv, dup, dd, defer ? &cs : nullptr)) {
        if (gl == 0) push_job(a, kJobTask, t, c, cs);
        return;
    }
    task_complete<G>(a, pt, i, slot, s, mode, c, conv, dup, gl, mask, leader);
}

// Certification job j: the FP64 residual pass of a deferred seed, the rest of its solve, and
// the completion of its point or task.
template <int G>
__device__ void job_step(Group<G> &grp, const SolveArgs &a, long long j, int gl, unsigned mask, int leader,
                         Counters &cnt) {
    const SolveOpts &o = a.opts;
    int ready = 0;
    if (gl == 0) ready = wait_ready(&a.job_ready[j], o.ready_polls);
    ready = __shfl_sync(mask, ready, leader);
    if (!ready) {
        cnt.v[kStatWaitTimeouts] += 1;
        return;
    }
    __threadfence();
    long long t;
    int kind;
    Candidate c;
    CertState cs;
    load_job(&a.jobs[j], t, kind, c, cs);
    bool conv = false;
    if (kind == kJobPoint) {
        PointIn pt;
        load_point(a, t, pt);
        double x0[5];
        for (int k = 0; k < 5; ++k) x0[k] = a.point_seeds[5 * t + k];
        PublishedRoots own{nullptr, nullptr, 0, 0, nullptr, mask, leader, gl, qnan()};
        own.own.remember(cs.x32);
        grp.mixed_seed_finish(pt, x0, o, c, conv, own, cs);
        point_complete<G>(a, pt, t, x0, c, conv, gl, cnt);
    } else {
        int64_t slot, i;
        int s, mode;
        if (!task_slot(a, t, false, gl, mask, leader, cnt, slot, s, i, mode)) return;
        PointIn pt;
        load_point(a, i, pt);
        const double *row = table_row(a, pt, s);
        double x0[5], prior[5];
        for (int k = 0; k < 5; ++k) x0[k] = row[k];
        PublishedRoots dd = task_roots(a, slot, s, mode, prior, mask, leader, gl);
        dd.own.remember(cs.x32);
        grp.mixed_seed_finish(pt, x0, o, c, conv, dd, cs);
        task_complete<G>(a, pt, i, slot, s, mode, c, conv, false, gl, mask, leader);
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
        point_step(grp, a, t, gl, cnt, false);
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
// still list them), and sleep per poll (ns).  A group that gives up simply exits: the work
// listed later is taken by the groups still running, at the latest by the one that listed it.
constexpr unsigned kIdlePolls = 1u << 22;
constexpr unsigned kIdleSleepNs = 500;

// Take the next entry of a device queue whose length grows while the kernel runs (head <
// avail): CAS so that no index beyond the published length is ever taken.  -1 when none.
__device__ __forceinline__ long long take_bounded(long long *head, long long avail) {
    long long h = *(volatile const long long *)head;
    while (h < avail) {
        const long long old =
            (long long)atomicCAS((unsigned long long *)head, (unsigned long long)h, (unsigned long long)(h + 1));
        if (old == h) return h;
        h = old;
    }
    return -1;
}

// Per-point seeds and the tasks they list in one persistent launch.  A group takes, in this
// order: a listed (slot, seed) task not yet taken; the next point; a queued certification;
// and, when nothing is left while points are still in flight, waits for their work.
// Verification seeds thus start as soon as their point is listed and share the GPU with the
// remaining points, instead of forming a second launch whose elapsed time is set by its
// longest seeds.
// With cert_warps = K > 0 the first K warps of every block are certifying warps: they take
// only queued certifications (the FP64 residual pass of a seed whose float-float refinement
// is done, and the rest of that seed), and the other warps queue them instead of running the
// FP64 pass themselves.  The FP64 pipe -- about 2 FMA per clock per SM on the GB300 -- then
// has a steady supply of work beside the FP32-pipe Newton and float-float passes.  (Measured
// on the 256 x 256 x 9 scan: no faster than K = 0, the default; the autotuner tries 0..4.)
template <int G>
__global__ void __launch_bounds__(kFusedThreads, 1) mixed_fused_kernel(SolveArgs a) {
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
    const bool defer = a.cert_warps > 0;
    const bool certifier = defer && (int)(threadIdx.x >> 5) < a.cert_warps;
    unsigned idle = 0;
    while (true) {
        long long t = 0;
        int kind = 0;  // 1 task, 2 point, 3 certification, 0 nothing yet, -1 all work taken
        if (gl == 0) {
            // read "all points completed" before the queue lengths: every slot listed by then
            // is included in them
            const bool all_points = *(volatile const long long *)a.points_done >= a.n;
            __threadfence();
            const long long jobs = defer ? *(volatile const long long *)a.job_count : 0;
            if (certifier) {
                t = take_bounded(a.job_head, jobs);
                if (t >= 0) kind = 3;
            } else {
                t = take_bounded(a.queue2, *(volatile const long long *)a.list_count * S);
                if (t >= 0) kind = 1;
                // two passes over the points: first those in the verification region, whose
                // listed tasks then start early, then the rest (a point is taken in one pass
                // and skipped in the other)
                while (kind == 0 && *(volatile const long long *)a.queue < 2 * a.n) {
                    t = (long long)atomicAdd((unsigned long long *)a.queue, 1ull);
                    if (t >= 2 * a.n) break;
                    const int64_t i = t < a.n ? t : t - a.n;
                    PointIn pt;
                    load_point(a, i, pt);
                    const bool first = a.n_seeds > 0 && valid_point(pt) && verification_region(a.opts, pt, a.P.hbarc);
                    if ((t < a.n) == first) {
                        kind = 2;
                        t = i;
                    }
                }
                if (kind == 0 && defer) {
                    t = take_bounded(a.job_head, jobs);
                    if (t >= 0) kind = 3;
                }
            }
            if (kind == 0 && all_points) {
                // nothing left to take: done, unless tasks remain for a non-certifying warp
                const bool tasks_left = *(volatile const long long *)a.queue2 < *(volatile const long long *)a.list_count * S;
                if (!(certifier && tasks_left)) kind = -1;
            }
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
        if (kind == 1) task_step(grp, a, t, false, gl, mask, leader, cnt, defer);
        else if (kind == 2) point_step(grp, a, t, gl, cnt, defer);
        else job_step(grp, a, t, gl, mask, leader, cnt);
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
    mixed_fused_kernel<32><<<grid, kFusedThreads, smem, s>>>(a);
    return cudaGetLastError();
}

int solve_mixed_occupancy(int kernel, size_t smem) {
    int nb = 0;
    cudaError_t e;
    if (kernel == kMixedTasks)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, mixed_tasks_kernel<32>, kSolveThreads, smem);
    else if (kernel == kMixedFused)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, mixed_fused_kernel<32>, kFusedThreads, smem);
    else
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, mixed_points_kernel<32>, kSolveThreads, smem);
    return e == cudaSuccess ? nb : 0;
}

}  // namespace pnjl
