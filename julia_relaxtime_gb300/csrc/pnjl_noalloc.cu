// pnjl_noalloc.cu -- pnjl_solve_batch_noalloc: a batched solve that allocates nothing.
//
// Who needs it: callers that may not allocate device memory at the moment they solve --
// hosts whose device memory is owned by another allocator (a Julia or PyTorch memory pool
// that must account for every byte, and would be bypassed by a cudaMalloc here), and
// long-running services that reserve all memory at start-up so that no call can fail for
// lack of it later.  They pass device inputs and outputs; everything else the solve needs
// lives in one file-scope static device array declared below, so no call makes a context,
// cudaMalloc, cudaFree or any allocating library routine.
//
// Precision: only the plain FP64 path (PNJL_PREC_FP64).  The mixed-precision solver needs
// per-seed records, published roots and a certification queue that this fixed array does
// not hold, so opts->precision = PNJL_PREC_MIXED is rejected with PNJL_ERR_INVALID_ARGUMENT.
//
// The scratch is the same as pnjl_solve_batch_device's: per-(point, seed) candidate records
// and per-point completion counters of the MultiSeed selection, the work-queue head and the
// counters, plus the separable node tables and the seed tables.  Its size is fixed at
// compile time (PNJL_NOALLOC_MAX_TASKS tasks, about 6 MB); every GPU that loads the library
// holds it until the process exits.
#include <cstring>
#include <mutex>

#include "pnjl_host_common.h"
#include "pnjl_kernels.h"

namespace {

constexpr int64_t kMaxTasks = PNJL_NOALLOC_MAX_TASKS;
constexpr size_t kAlign = 256;
constexpr size_t round_up(size_t b) { return (b + kAlign - 1) & ~(kAlign - 1); }

// byte offsets inside the static array
constexpr size_t kCtrlOff = 0;  // kCtrlSlots x int64: queue head + counters
constexpr size_t kDoneOff = kCtrlOff + round_up(pnjl::kCtrlSlots * sizeof(long long));        // kMaxTasks x int
constexpr size_t kCandOff = kDoneOff + round_up(kMaxTasks * sizeof(int));       // kMaxTasks x CandRec
constexpr size_t kNodesOff = kCandOff + round_up(kMaxTasks * sizeof(pnjl::CandRec));
constexpr size_t kNodesF64 = 2 * (pnjl::kMaxPNodes + pnjl::kMaxTNodes);         // doubles
constexpr size_t kNodesF32Off = kNodesOff + round_up(kNodesF64 * sizeof(double));
constexpr size_t kSeedsOff = kNodesF32Off + round_up(kNodesF64 * sizeof(float)); // 2 x 16 x 5 doubles
constexpr size_t kScratchBytes = kSeedsOff + round_up(2 * 16 * 5 * sizeof(double));

}  // namespace

// The one static scratch array.  Host code must not use its name as an address: the name
// is a host-side stand-in; the device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;                          // serialises set-up and the host-side tables
unsigned char *g_scratch_addr[kMaxDevices];  // device address of g_noalloc_scratch per device
bool g_ready[kMaxDevices];
// host copies of the node tables of the last (p_num, t_num, p_max)
int g_p = 0, g_t = 0;
double g_pmax = 0.0;
double g_tab[kNodesF64];
float g_tabf[kNodesF64];

// Set-up, once per device, with that device current: the device address of the array.
int scratch_for_current_device(unsigned char **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PNJL_ERR_CUDA;
    if (!g_ready[dev]) {
        void *ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || ptr == nullptr) return PNJL_ERR_CUDA;
        g_scratch_addr[dev] = (unsigned char *)ptr;
        g_ready[dev] = true;
    }
    *out = g_scratch_addr[dev];
    return PNJL_OK;
}

void node_tables(int p_num, int t_num, double p_max) {
    if (p_num == g_p && t_num == g_t && p_max == g_pmax) return;
    double xp[pnjl::kMaxPNodes], wp[pnjl::kMaxPNodes], xc[pnjl::kMaxTNodes], wc[pnjl::kMaxTNodes];
    pnjl::gauss_legendre_into(p_num, 0.0, p_max, xp, wp);
    pnjl::gauss_legendre_into(t_num, 0.0, 1.0, xc, wc);
    pnjl::separable_tables(p_num, t_num, xp, wp, xc, wc, g_tab, g_tabf);
    g_p = p_num;
    g_t = t_num;
    g_pmax = p_max;
}

}  // namespace

extern "C" int pnjl_solve_batch_noalloc(const pnjl_params *params, int32_t p_num, int32_t t_num, double p_max,
                                        int64_t n, const double *d_T, const double *d_mu_u, const double *d_mu_d,
                                        const double *d_mu_s, const double *d_xi, const pnjl_solve_opts *opts,
                                        pnjl_result_soa *d_out, void *stream) {
    if (!params || !d_out) return PNJL_ERR_INVALID_ARGUMENT;
    const char *msg = "";
    if (pnjl::validate_opts(opts, &msg) != PNJL_OK) return PNJL_ERR_INVALID_ARGUMENT;
    if (opts->verify_map) return PNJL_ERR_INVALID_ARGUMENT;  // no device copy without an allocation
    if (opts->precision != PNJL_PREC_FP64) return PNJL_ERR_INVALID_ARGUMENT;  // FP64 kernel only
    if (p_num < 1 || p_num > pnjl::kMaxPNodes || t_num < 1 || t_num > pnjl::kMaxTNodes || !(p_max > 0.0))
        return PNJL_ERR_INVALID_ARGUMENT;
    if (n < 0 || (n > 0 && (!d_T || !d_mu_u || !d_mu_d || !d_mu_s || !d_xi))) return PNJL_ERR_INVALID_ARGUMENT;
    const bool table_mode = opts->seed_mode == PNJL_SEEDS_TABLE;
    const int64_t tasks = table_mode ? n * (int64_t)opts->n_seeds : n;
    if (n > kMaxTasks || tasks > kMaxTasks) return PNJL_ERR_TOO_LARGE;
    if (n == 0) return PNJL_OK;
    cudaStream_t s = (cudaStream_t)stream;

    std::lock_guard<std::mutex> lock(g_mu);
    unsigned char *base = nullptr;
    if (scratch_for_current_device(&base) != PNJL_OK) return PNJL_ERR_CUDA;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return PNJL_ERR_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return PNJL_ERR_CUDA;

    node_tables(p_num, t_num, p_max);
    const int m = 2 * (p_num + t_num);
    double *d_nodes = (double *)(base + kNodesOff);
    float *d_nodes_f = (float *)(base + kNodesF32Off);
    double *d_seeds = (double *)(base + kSeedsOff);
    long long *d_ctrl = (long long *)(base + kCtrlOff);
    int *d_done = (int *)(base + kDoneOff);
    pnjl::CandRec *d_cand = (pnjl::CandRec *)(base + kCandOff);
    // the array keeps the previous call's contents: reset the counters, reload the tables
    if (cudaMemcpyAsync(d_nodes, g_tab, m * sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(d_nodes_f, g_tabf, m * sizeof(float), cudaMemcpyHostToDevice, s) != cudaSuccess)
        return PNJL_ERR_CUDA;
    const bool has_table = opts->n_seeds > 0 && opts->seed_table;
    if (has_table) {
        if (cudaMemcpyAsync(d_seeds, opts->seed_table, opts->n_seeds * 5 * sizeof(double), cudaMemcpyHostToDevice,
                            s) != cudaSuccess)
            return PNJL_ERR_CUDA;
        if (opts->seed_table_hot &&
            cudaMemcpyAsync(d_seeds + 80, opts->seed_table_hot, opts->n_seeds * 5 * sizeof(double),
                            cudaMemcpyHostToDevice, s) != cudaSuccess)
            return PNJL_ERR_CUDA;
    }
    if (cudaMemsetAsync(d_ctrl, 0, pnjl::kCtrlSlots * sizeof(long long), s) != cudaSuccess) return PNJL_ERR_CUDA;
    if (table_mode && cudaMemsetAsync(d_done, 0, (size_t)n * sizeof(int), s) != cudaSuccess) return PNJL_ERR_CUDA;

    pnjl::SolveArgs a{};
    a.P = pnjl::dev_params(*params);
    a.nodes.p_num = p_num;
    a.nodes.t_num = t_num;
    a.nodes.p2 = d_nodes;
    a.nodes.A = d_nodes + p_num;
    a.nodes.c2 = d_nodes + 2 * p_num;
    a.nodes.B = d_nodes + 2 * p_num + t_num;
    a.nodes.p2f = d_nodes_f;
    a.nodes.Af = d_nodes_f + p_num;
    a.nodes.c2f = d_nodes_f + 2 * p_num;
    a.nodes.Bf = d_nodes_f + 2 * p_num + t_num;
    a.n = n;
    a.T = d_T; a.mu_u = d_mu_u; a.mu_d = d_mu_d; a.mu_s = d_mu_s; a.xi = d_xi;
    a.seed_mode = opts->seed_mode;
    a.n_seeds = has_table ? opts->n_seeds : 0;
    a.seed_table = d_seeds;
    a.seed_table_hot = (has_table && opts->seed_table_hot) ? d_seeds + 80 : nullptr;
    a.hot_T_MeV = opts->hot_T_MeV;
    a.point_seeds = opts->point_seeds;
    pnjl::fill_solve_opts(opts, a.opts);
    a.out = *d_out;
    a.cand = d_cand;
    a.done = d_done;
    a.queue = d_ctrl;
    a.stats = d_ctrl + 1;
    const size_t smem = pnjl::node_smem_bytes(p_num, t_num);
    int occ = pnjl::solve_kernel_occupancy(32, smem);
    if (occ < 1) occ = 1;
    const int64_t groups_per_block = pnjl::kSolveThreads / 32;
    int64_t grid = (int64_t)sms * occ;
    const int64_t need = (tasks + groups_per_block - 1) / groups_per_block;
    if (need < grid) grid = need;
    if (pnjl::launch_solve(a, 32, (int)grid, smem, s) != cudaSuccess) return PNJL_ERR_CUDA;
    return PNJL_OK;
}
