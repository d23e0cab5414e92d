// pnjl_kernels.h -- launch interface between the C ABI (pnjl_capi.cu) and the kernels.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/pnjl_cuda.h"
#include "pnjl_device.cuh"

namespace pnjl {

static constexpr int kSolveThreads = 256;
// threads per block of the fused mixed kernel (one block per SM)
static constexpr int kFusedThreads = 256;

// Separable node tables on the device (FP64 and an FP32 copy).
struct KernelNodes {
    const double *p2, *A, *c2, *B;
    const float *p2f, *Af, *c2f, *Bf;
    // float-float low parts of the FP32 tables (same layout) and the float-float exp tables
    // (kExpTableFloats); null where a kernel has no float-float pass
    const float *lo, *expt;
    int p_num, t_num;
};

// Scratch record of one (point, seed) task in MultiSeed mode (176 bytes).
struct CandRec {
    double x[5];
    double residual_norm, omega, entropy;
    double rho[3], nq[3], naq[3];
    int iterations, flags;
};

// State of a seed whose FP64 certification is deferred (see Group::mixed_solve_seed): its
// FP32 root, FP32 iterations, refinement steps so far, whether the candidate's thermo fields
// belong to its state.
struct CertState {
    double x32[5];
    int it32, steps, th_valid, unstable;
};

// Scratch record of a deferred seed, from the warp that refined it to a certifying warp:
// the item (a point of the per-point queue or a (slot, seed) task), its CertState and the
// candidate (state, thermo fields, flags: bit 0 f_converged, 1 exception, 2 phys).
enum JobKind { kJobTask = 1, kJobPoint = 2 };
struct CertJob {
    long long t;
    int kind, flags, iterations, pad;
    CertState cs;
    double x[5], residual_norm, omega, entropy, rho[3], nq[3], naq[3];
};

// Counter slots of SolveArgs::stats
enum StatSlot {
    kStatPasses64 = 0, kStatEvalsNewton64, kStatEvalsThermo64, kStatSeeds, kStatTrRuns, kStatMsFallbacks,
    kStatPasses32, kStatEvals32, kStatEvalsGrad64, kStatEvalsGradThermo64, kStatRescue64, kStatEvalsThermo32,
    kStatPruned, kStatEvalsFF, kStatEvalsFFThermo, kStatWaitTimeouts, kStatEvalsFFGradThermo, kStatCount
};

struct SolveArgs {
    DevParams P;
    KernelNodes nodes;
    int64_t n;
    const double *T, *mu_u, *mu_d, *mu_s, *xi;
    int seed_mode, n_seeds;
    const double *seed_table;     // device [n_seeds*5]
    const double *seed_table_hot; // device or null
    double hot_T_MeV;
    const double *point_seeds;    // device [n*5]
    SolveOpts opts;
    pnjl_result_soa out;          // device pointers
    CandRec *cand;                // scratch: FP64 kernel [n*n_seeds]; mixed kernels [n*(n_seeds+1)]
    int *done;                    // scratch [n], zeroed before the launch
    long long *queue;             // device work-queue head (zeroed before the launch)
    long long *stats;             // device counters [kStatCount]
    // mixed-precision task kernel (zeroed before the launch where noted)
    double *roots;                // [n*n_seeds*5] FP32 roots published per (slot, seed)
    int *root_flag;               // [n*n_seeds] state of roots[slot, seed]: none / pending / usable (zeroed)
    long long *list;              // [n] points deferred by the per-point kernel
    int *list_mode;               // [n] kListVerify / kListFallback, stored + 1 once the slot's
                                  // point and record are written (zeroed: 0 = not yet)
    long long *list_count;        // entries in list (zeroed)
    long long *queue2;            // work-queue head of the task kernel (zeroed)
    long long *points_done;       // fused kernel: points completed (written or listed) (zeroed)
    // fused kernel with certifying warps (cert_warps > 0 per block)
    int cert_warps;
    CertJob *jobs;                // [n * (n_seeds + 1)] deferred seeds
    int *job_ready;               // [n * (n_seeds + 1)] 1 once jobs[j] is written (zeroed)
    int *anchor_state;            // [n] seed 0's verdict: 0 pending, 1 certified usable, 2 not (zeroed)
    double *anchor_omega;         // [n] seed 0's Omega once anchor_state is 1
    long long *job_count;         // jobs reserved (zeroed)
    long long *job_head;          // jobs taken (zeroed)
};

// Modes of a slot of the mixed task kernel: min-Omega over all seeds (MultiSeed table mode);
// a converged per-point solution checked against the first verify_seeds seeds; a per-point
// seed that failed, replaced by the MultiSeed solve (ImplicitSolver.jl:306-327).
// the control block of a context: queue head, counters, list length, task queue head,
// finished points of the fused kernel
constexpr int kCtrlSlots = 80;
// per-chunk queue heads of the pipelined mixed per-point solve: queue, list length, task queue
constexpr int kMaxPipelineChunks = 16;
constexpr int kChunkCtrlBase = 24;
static_assert(1 + kStatCount + 5 <= kChunkCtrlBase, "control block too small");
// certifying warps per block of the fused kernel (pnjl_set_cert_warps), by default
constexpr int kDefaultCertWarps = 0;
static_assert(kChunkCtrlBase + 3 * kMaxPipelineChunks <= kCtrlSlots, "chunk control slots");

enum ListMode { kListFull = 0, kListVerify = 1, kListFallback = 2 };

struct EvalArgs {
    DevParams P;
    KernelNodes nodes;
    int64_t n;
    const double *x, *T, *mu_u, *mu_d, *mu_s, *xi;
    double *omega, *grad, *hess;
    pnjl_result_soa out;
};

// build_K_data per point (pnjl_kdata.cu): one thread per point, node table in shared memory
struct KDataArgs {
    double Lambda, G, K;
    int p_num;
    const double *p, *w;  // device Gauss-Legendre nodes and weights on [0, p_max]
    int64_t n;
    const double *T, *mu_u, *mu_s, *masses, *x;
    pnjl_kdata_soa out;
};
cudaError_t launch_kdata(const KDataArgs &a, int sm_count, cudaStream_t s);

// implicit derivatives of solved states (pnjl_deriv.cu): one warp per point
struct DerivArgs {
    DevParams P;
    KernelNodes nodes;
    int64_t n;
    const double *x, *T, *mu_u, *mu_d, *mu_s, *xi;
    pnjl_deriv_soa out;
};
cudaError_t launch_deriv(const DerivArgs &a, int grid, size_t smem, cudaStream_t s);

size_t node_smem_bytes(int p_num, int t_num);
cudaError_t launch_solve(const SolveArgs &a, int group, int grid, size_t smem, cudaStream_t s);
// Mixed precision: per-point mode launches the fused kernel (points and the tasks they defer
// in one launch), or the per-point kernel and then the task kernel over the points it
// deferred; table mode launches the task kernel alone.
cudaError_t launch_mixed_points(const SolveArgs &a, int grid, size_t smem, cudaStream_t s);
cudaError_t launch_mixed_tasks(const SolveArgs &a, int grid, size_t smem, cudaStream_t s);
cudaError_t launch_mixed_fused(const SolveArgs &a, int grid, size_t smem, cudaStream_t s);
enum MixedKernel { kMixedPoints = 0, kMixedTasks = 1, kMixedFused = 2 };
int solve_mixed_occupancy(int kernel, size_t smem);
cudaError_t launch_eval(const EvalArgs &a, int mode, int grid, size_t smem, cudaStream_t s);  // 0 FP64, 1 FP32, 2 ff
int solve_kernel_occupancy(int group, size_t smem);

}  // namespace pnjl
