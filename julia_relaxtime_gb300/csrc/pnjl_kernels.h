// pnjl_kernels.h -- launch interface between the C ABI (pnjl_capi.cu) and the kernels.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/pnjl_cuda.h"
#include "pnjl_device.cuh"

namespace pnjl {

static constexpr int kSolveThreads = 256;

struct KernelNodes {
    const double *p2, *pc2, *w;
    const float *p2f, *pc2f, *wf;
    int n;
};

struct SolveArgs {
    DevParams P;
    KernelNodes nodes;
    bool stage_nodes;
    int64_t n;
    const double *T, *mu_u, *mu_d, *mu_s, *xi;
    int seed_mode, n_seeds;
    const double *seed_table;     // device [n_seeds*5]
    const double *seed_table_hot; // device or null
    double hot_T_MeV;
    const double *point_seeds;    // device [n*5]
    SolveOpts opts;
    pnjl_result_soa out;          // device pointers
    long long *queue;             // device work-queue head (zeroed before the launch)
    long long *stats;             // device counters [8]
};

struct EvalArgs {
    DevParams P;
    KernelNodes nodes;
    bool stage_nodes;
    int64_t n;
    const double *x, *T, *mu_u, *mu_d, *mu_s, *xi;
    double *omega, *grad, *hess;
    pnjl_result_soa out;
};

size_t node_smem_bytes(int n, bool fp32_too);
cudaError_t launch_solve(const SolveArgs &a, int group, int grid, size_t smem, cudaStream_t s);
cudaError_t launch_eval(const EvalArgs &a, bool fp32, int grid, size_t smem, cudaStream_t s);
int solve_kernel_occupancy(int group, size_t smem);

}  // namespace pnjl
