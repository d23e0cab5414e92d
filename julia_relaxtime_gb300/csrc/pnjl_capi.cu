// pnjl_capi.cu -- the extern "C" boundary of libpnjl_cuda (declared in include/pnjl_cuda.h).
//
// Owns the per-context state: device, stream, model constants, node meshes (FP64 and an
// FP32 copy), a growable device workspace for the host-pointer entry points, the work-queue
// head and the counters.  Every entry point returns a PNJL_* code and records a message
// for pnjl_last_error(); no C++ exception crosses the boundary.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "pnjl_host_common.h"
#include "pnjl_kernels.h"
#include "pnjl_mlp.h"

struct pnjl_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev_mid = nullptr;
    long long *d_ctrl_snap = nullptr;  // counters after the first kernel of a two-kernel solve
    bool split_last = false;           // the last solve ran two kernels (ev_mid, d_ctrl_snap valid)
    pnjl_params params{};
    pnjl::DevParams dp{};
    // nodes
    int p_num = 0, t_num = 0;
    double p_max = 0.0;
    std::vector<double> p_mesh, c_mesh, coef;
    double *d_nodes = nullptr;  // p2[p] | A[p] | c2[t] | B[t]
    float *d_nodes_f = nullptr; // the same in FP32
    // control block (kCtrlSlots): [0] queue head, [1..kStatCount] counters, list length, task queue
    long long *d_ctrl = nullptr;
    double *d_seed_tables = nullptr; // 2 * 16 * 5
    unsigned char *d_vmap = nullptr;  // device copy of the verification map
    size_t vmap_cap = 0;
    // workspace for the host entry points
    unsigned char *d_ws = nullptr;
    size_t ws_cap = 0;
    // pinned host mirror of the workspace for the host-array solves (one DMA each way)
    unsigned char *h_stage = nullptr;
    size_t stage_cap = 0;
    // K data: Gauss-Legendre nodes and weights of the last (p_num, p_max) on the device
    double *d_kd_nodes = nullptr;  // p[kMaxPNodes] | w[kMaxPNodes]
    int kd_p_num = 0;
    double kd_p_max = 0.0;
    // solver scratch: candidate records and per-point completion counters (MultiSeed mode)
    unsigned char *d_scratch = nullptr;
    size_t scratch_cap = 0;
    // tuning
    int group = 32;
    int blocks_per_sm = 0;  // 0 = occupancy maximum
    int pipeline_chunks = 0;  // mixed per-point solves: chunks over two streams (0 = automatic)
    int cert_warps = pnjl::kDefaultCertWarps;  // fused kernel: certifying warps per block
    unsigned ready_polls = pnjl::kReadyPollsDefault;      // bounds of the fused kernel's waits
    unsigned verdict_polls = pnjl::kVerdictPollsDefault;  // (pnjl_set_wait_limits)
    cudaStream_t stream2 = nullptr;  // second stream of the chunk pipeline
    cudaEvent_t ev_chunk[pnjl::kMaxPipelineChunks] = {};
    cudaEvent_t ev_join = nullptr;
    pnjl_stats stats{};
    std::string err;
    // learned seed
    struct Mlp {
        bool ready = false, scaled = false, trained = false;
        float *params = nullptr;  // master | grad | adam m | adam v  (4 x kParamCount)
        __nv_bfloat16 *wb = nullptr;
        long long *step = nullptr;
        float *loss = nullptr;
        float *x = nullptr, *y = nullptr;
        float *partial = nullptr;  // gradient slots [kMaxGradSlots][kParamCount], then slot losses
        int *perm = nullptr;       // epoch permutations [epochs][n]
        size_t cap = 0, perm_cap = 0;
        double *seeds = nullptr;  // per-point seeds of pnjl_solve_batch_learned*
        size_t seeds_cap = 0;
        pnjl::Scaling sc{};
    } mlp;
};

namespace {

int fail(pnjl_ctx *ctx, int code, const std::string &msg) {
    if (ctx) ctx->err = msg;
    return code;
}

int cuda_fail(pnjl_ctx *ctx, cudaError_t e, const char *what) {
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return fail(ctx, PNJL_ERR_CUDA, m);
}

#define PNJL_CUDA_TRY(ctx, call)                                   \
    do {                                                           \
        cudaError_t _e = (call);                                   \
        if (_e != cudaSuccess) return cuda_fail((ctx), _e, #call); \
    } while (0)

void gauss_legendre(int n, double a, double b, std::vector<double> &x, std::vector<double> &w) {
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    pnjl::gauss_legendre_into(n, a, b, x.data(), w.data());
}

template <typename T>
T *carve(unsigned char *&p, size_t count) {
    T *r = reinterpret_cast<T *>(p);
    size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
    p += bytes;
    return r;
}
size_t carve_size(size_t count, size_t elem) { return (count * elem + 255) & ~size_t(255); }

int ensure_ws(pnjl_ctx *ctx, size_t bytes) {
    if (bytes <= ctx->ws_cap) return PNJL_OK;
    if (ctx->d_ws) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(ctx->d_ws);
        ctx->d_ws = nullptr;
        ctx->ws_cap = 0;
    }
    size_t cap = bytes + bytes / 4;
    cudaError_t e = cudaMalloc(&ctx->d_ws, cap);
    if (e != cudaSuccess) {
        ctx->d_ws = nullptr;
        return fail(ctx, PNJL_ERR_OUT_OF_MEMORY, std::string("workspace allocation failed: ") + cudaGetErrorString(e));
    }
    ctx->ws_cap = cap;
    return PNJL_OK;
}

// Pinned staging of at least `bytes`; false (and the caller copies pageable memory
// directly) when pinned memory is not available.
bool ensure_stage(pnjl_ctx *ctx, size_t bytes) {
    if (bytes <= ctx->stage_cap) return true;
    if (ctx->h_stage) {
        cudaStreamSynchronize(ctx->stream);
        cudaFreeHost(ctx->h_stage);
        ctx->h_stage = nullptr;
        ctx->stage_cap = 0;
    }
    const size_t cap = bytes + bytes / 4;
    if (cudaHostAlloc(&ctx->h_stage, cap, cudaHostAllocDefault) != cudaSuccess) {
        ctx->h_stage = nullptr;
        cudaGetLastError();  // clear the failed call
        return false;
    }
    ctx->stage_cap = cap;
    return true;
}

pnjl::KernelNodes kernel_nodes(const pnjl_ctx *ctx) {
    pnjl::KernelNodes kn;
    const int np = ctx->p_num, nt = ctx->t_num;
    kn.p_num = np;
    kn.t_num = nt;
    kn.p2 = ctx->d_nodes;
    kn.A = ctx->d_nodes + np;
    kn.c2 = ctx->d_nodes + 2 * np;
    kn.B = ctx->d_nodes + 2 * np + nt;
    kn.p2f = ctx->d_nodes_f;
    kn.Af = ctx->d_nodes_f + np;
    kn.c2f = ctx->d_nodes_f + 2 * np;
    kn.Bf = ctx->d_nodes_f + 2 * np + nt;
    kn.lo = ctx->d_nodes_f + 2 * (np + nt);
    kn.expt = ctx->d_nodes_f + 4 * (np + nt);
    return kn;
}

int ensure_scratch(pnjl_ctx *ctx, size_t bytes) {
    if (bytes <= ctx->scratch_cap) return PNJL_OK;
    if (ctx->d_scratch) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(ctx->d_scratch);
        ctx->d_scratch = nullptr;
        ctx->scratch_cap = 0;
    }
    size_t cap = bytes + bytes / 4;
    cudaError_t e = cudaMalloc(&ctx->d_scratch, cap);
    if (e != cudaSuccess) {
        ctx->d_scratch = nullptr;
        return fail(ctx, PNJL_ERR_OUT_OF_MEMORY, std::string("scratch allocation failed: ") + cudaGetErrorString(e));
    }
    ctx->scratch_cap = cap;
    return PNJL_OK;
}

int check_opts(pnjl_ctx *ctx, const pnjl_solve_opts *o) {
    const char *msg = "";
    const int rc = pnjl::validate_opts(o, &msg);
    return rc ? fail(ctx, rc, msg) : PNJL_OK;
}

int grid_for(const pnjl_ctx *ctx, int group, size_t smem, int64_t n) {
    int occ = pnjl::solve_kernel_occupancy(group, smem);
    if (occ < 1) occ = 1;
    int bps = ctx->blocks_per_sm > 0 ? std::min(ctx->blocks_per_sm, occ) : occ;
    const int64_t groups_per_block = pnjl::kSolveThreads / group;
    int64_t need = (n + groups_per_block - 1) / groups_per_block;
    int64_t g = (int64_t)ctx->sm_count * bps;
    if (need < g) g = need;
    if (g < 1) g = 1;
    return (int)g;
}


pnjl::MlpDev mlp_dev(pnjl_ctx *ctx) {
    pnjl::MlpDev m;
    m.master = ctx->mlp.params;
    m.grad = ctx->mlp.params + pnjl::kParamCount;
    m.adam_m = ctx->mlp.params + 2 * pnjl::kParamCount;
    m.adam_v = ctx->mlp.params + 3 * pnjl::kParamCount;
    const int H = pnjl::mlp::H, IN = pnjl::mlp::IN;
    m.w1b = ctx->mlp.wb;
    m.w2b = ctx->mlp.wb + H * IN;
    m.w3b = m.w2b + H * H;
    m.w4b = m.w3b + H * H;
    m.partial = ctx->mlp.partial;
    m.loss_part = ctx->mlp.partial + (size_t)pnjl::kMaxGradSlots * pnjl::kParamCount;
    return m;
}

int mlp_require(pnjl_ctx *ctx, bool need_scaling) {
    if (!ctx->mlp.ready) return fail(ctx, PNJL_ERR_NOT_TRAINED, "call pnjl_mlp_init first");
    if (need_scaling && !ctx->mlp.scaled) return fail(ctx, PNJL_ERR_NOT_TRAINED, "call pnjl_mlp_set_scaling first");
    return PNJL_OK;
}

int mlp_ensure_data(pnjl_ctx *ctx, size_t n) {
    if (n <= ctx->mlp.cap) return PNJL_OK;
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->mlp.x);
    cudaFree(ctx->mlp.y);
    ctx->mlp.x = nullptr; ctx->mlp.y = nullptr; ctx->mlp.cap = 0;
    if (cudaMalloc(&ctx->mlp.x, n * pnjl::mlp::IN * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&ctx->mlp.y, n * pnjl::mlp::OUT * sizeof(float)) != cudaSuccess)
        return fail(ctx, PNJL_ERR_OUT_OF_MEMORY, "MLP data allocation failed");
    ctx->mlp.cap = n;
    return PNJL_OK;
}

int mlp_ensure_perm(pnjl_ctx *ctx, size_t count) {
    if (count <= ctx->mlp.perm_cap) return PNJL_OK;
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->mlp.perm);
    ctx->mlp.perm = nullptr;
    ctx->mlp.perm_cap = 0;
    if (cudaMalloc(&ctx->mlp.perm, count * sizeof(int)) != cudaSuccess)
        return fail(ctx, PNJL_ERR_OUT_OF_MEMORY, "MLP permutation allocation failed");
    ctx->mlp.perm_cap = count;
    return PNJL_OK;
}

// splitmix64: deterministic host RNG for the initial weights and the epoch shuffles
uint64_t splitmix64(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
double uniform01(uint64_t &s) { return (splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

}  // namespace

extern "C" {

int pnjl_params_default(pnjl_params *out) {
    if (!out) return PNJL_ERR_INVALID_ARGUMENT;
    const double hbarc = 197.327;
    out->hbarc_MeV_fm = hbarc;
    out->Lambda = 602.3 / hbarc;
    out->m_ud0 = 5.5 / hbarc;
    out->m_s0 = 140.7 / hbarc;
    out->G = 1.835 / (out->Lambda * out->Lambda);
    out->K = 12.36 / std::pow(out->Lambda, 5);
    out->T0 = 210.0 / hbarc;
    out->a0 = 3.51;
    out->a1 = -2.47;
    out->a2 = 15.2;
    out->b3 = -1.75;
    out->N_color = 3.0;
    out->rho0 = 0.16;
    return PNJL_OK;
}

int pnjl_init(const pnjl_params *params, int device, pnjl_ctx **out) {
    if (!out) return PNJL_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    pnjl_ctx *ctx = new (std::nothrow) pnjl_ctx();
    if (!ctx) return PNJL_ERR_OUT_OF_MEMORY;
    if (params) ctx->params = *params;
    else pnjl_params_default(&ctx->params);
    const pnjl_params &p = ctx->params;
    ctx->dp = pnjl::dev_params(p);
    ctx->device = device;
    int rc = PNJL_OK;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev_mid);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream2, cudaStreamNonBlocking);
    for (int k = 0; k < pnjl::kMaxPipelineChunks && e == cudaSuccess; ++k)
        e = cudaEventCreateWithFlags(&ctx->ev_chunk[k], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_ctrl, pnjl::kCtrlSlots * sizeof(long long));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_ctrl_snap, pnjl::kCtrlSlots * sizeof(long long));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->d_seed_tables, 2 * 16 * 5 * sizeof(double));
    if (e != cudaSuccess) {
        std::fprintf(stderr, "pnjl_init: %s\n", cudaGetErrorString(e));
        rc = PNJL_ERR_CUDA;
        pnjl_destroy(ctx);
        return rc;
    }
    *out = ctx;
    return PNJL_OK;
}

int pnjl_destroy(pnjl_ctx *ctx) {
    if (!ctx) return PNJL_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->d_nodes);
    cudaFree(ctx->d_nodes_f);
    cudaFree(ctx->d_ctrl);
    cudaFree(ctx->d_seed_tables);
    cudaFree(ctx->d_vmap);
    cudaFree(ctx->d_ws);
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    cudaFree(ctx->d_scratch);
    cudaFree(ctx->d_kd_nodes);
    cudaFree(ctx->mlp.params);
    cudaFree(ctx->mlp.wb);
    cudaFree(ctx->mlp.step);
    cudaFree(ctx->mlp.loss);
    cudaFree(ctx->mlp.x);
    cudaFree(ctx->mlp.y);
    cudaFree(ctx->mlp.perm);
    cudaFree(ctx->mlp.partial);
    cudaFree(ctx->mlp.seeds);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->ev_mid) cudaEventDestroy(ctx->ev_mid);
    for (int k = 0; k < pnjl::kMaxPipelineChunks; ++k)
        if (ctx->ev_chunk[k]) cudaEventDestroy(ctx->ev_chunk[k]);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->stream2) cudaStreamDestroy(ctx->stream2);
    cudaFree(ctx->d_ctrl_snap);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return PNJL_OK;
}

const char *pnjl_last_error(const pnjl_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

// Device node tables of one quadrature (p_num x t_num, p in [0, p_max]): FP64 separable
// tables and the FP32 hi | float-float lo | float-float exp tables.
static void node_tables_host(int p_num, int t_num, double p_max, std::vector<double> &h, std::vector<float> &hf) {
    std::vector<double> xp, wp, xc, wc;
    gauss_legendre(p_num, 0.0, p_max, xp, wp);
    gauss_legendre(t_num, 0.0, 1.0, xc, wc);
    const int m = 2 * (p_num + t_num);
    h.assign(m, 0.0);
    hf.assign(2 * m + pnjl::kExpTableFloats, 0.0f);
    pnjl::separable_tables(p_num, t_num, xp.data(), wp.data(), xc.data(), wc.data(), h.data(), hf.data(),
                           hf.data() + m);
    pnjl::ff_exp_tables(hf.data() + 2 * m);
}

static pnjl::KernelNodes kernel_nodes_of(const double *d, const float *f, int np, int nt) {
    pnjl::KernelNodes kn;
    kn.p_num = np;
    kn.t_num = nt;
    kn.p2 = d; kn.A = d + np; kn.c2 = d + 2 * np; kn.B = d + 2 * np + nt;
    kn.p2f = f; kn.Af = f + np; kn.c2f = f + 2 * np; kn.Bf = f + 2 * np + nt;
    kn.lo = f + 2 * (np + nt);
    kn.expt = f + 4 * (np + nt);
    return kn;
}

int pnjl_set_nodes(pnjl_ctx *ctx, int32_t p_num, int32_t t_num, double p_max) {
    if (!ctx) return PNJL_ERR_INVALID_ARGUMENT;
    if (p_num < 1 || p_num > pnjl::kMaxPNodes || t_num < 1 || t_num > pnjl::kMaxTNodes || !(p_max > 0.0))
        return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "node counts out of range (1..512 x 1..64, p_max > 0)");
    cudaSetDevice(ctx->device);
    std::vector<double> xp, wp, xc, wc;
    gauss_legendre(p_num, 0.0, p_max, xp, wp);
    gauss_legendre(t_num, 0.0, 1.0, xc, wc);
    const int n = p_num * t_num;
    ctx->p_mesh.resize(n);
    ctx->c_mesh.resize(n);
    ctx->coef.resize(n);
    const double fourpi2 = (2.0 * M_PI) * (2.0 * M_PI);
    for (int it = 0; it < t_num; ++it)
        for (int ip = 0; ip < p_num; ++ip) {
            const int k = ip + p_num * it;  // column-major like Integrals.jl:87-97
            ctx->p_mesh[k] = xp[ip];
            ctx->c_mesh[k] = xc[it];
            ctx->coef[k] = (wp[ip] * (wc[it] * 2.0)) * (xp[ip] * xp[ip]) / fourpi2;
        }
    // separable device tables: p2[p] | A[p] = w_p p^2/(2 pi)^2 | c2[t] | B[t] = 2 w_c
    // FP32 device tables: hi parts | float-float lo parts | float-float exp tables
    const int m = 2 * (p_num + t_num);
    std::vector<double> h(m);
    std::vector<float> hf(2 * m + pnjl::kExpTableFloats);
    pnjl::separable_tables(p_num, t_num, xp.data(), wp.data(), xc.data(), wc.data(), h.data(), hf.data(),
                           hf.data() + m);
    pnjl::ff_exp_tables(hf.data() + 2 * m);
    PNJL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->d_nodes);
    cudaFree(ctx->d_nodes_f);
    ctx->d_nodes = nullptr;
    ctx->d_nodes_f = nullptr;
    PNJL_CUDA_TRY(ctx, cudaMalloc(&ctx->d_nodes, m * sizeof(double)));
    PNJL_CUDA_TRY(ctx, cudaMalloc(&ctx->d_nodes_f, hf.size() * sizeof(float)));
    PNJL_CUDA_TRY(ctx, cudaMemcpy(ctx->d_nodes, h.data(), m * sizeof(double), cudaMemcpyHostToDevice));
    PNJL_CUDA_TRY(ctx, cudaMemcpy(ctx->d_nodes_f, hf.data(), hf.size() * sizeof(float), cudaMemcpyHostToDevice));
    ctx->p_num = p_num;
    ctx->t_num = t_num;
    ctx->p_max = p_max;
    return PNJL_OK;
}

int pnjl_get_nodes(const pnjl_ctx *ctx, double *p_mesh, double *c_mesh, double *coef) {
    if (!ctx) return PNJL_ERR_INVALID_ARGUMENT;
    if (ctx->p_num == 0) return PNJL_ERR_NO_NODES;
    const size_t n = ctx->p_mesh.size();
    if (p_mesh) std::memcpy(p_mesh, ctx->p_mesh.data(), n * sizeof(double));
    if (c_mesh) std::memcpy(c_mesh, ctx->c_mesh.data(), n * sizeof(double));
    if (coef) std::memcpy(coef, ctx->coef.data(), n * sizeof(double));
    return PNJL_OK;
}

static int eval_common(pnjl_ctx *ctx, int64_t n, const double *x, const double *T, const double *mu_u,
                       const double *mu_d, const double *mu_s, const double *xi, int32_t precision, double *omega,
                       double *grad, double *hess, pnjl_result_soa *out) {
    if (!ctx) return PNJL_ERR_INVALID_ARGUMENT;
    if (ctx->p_num == 0) return fail(ctx, PNJL_ERR_NO_NODES, "call pnjl_set_nodes first");
    if (n < 0 || (n > 0 && (!x || !T || !mu_u || !mu_d || !mu_s || !xi)))
        return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "null input array");
    if (precision != PNJL_PREC_FP64 && precision != PNJL_PREC_MIXED && precision != PNJL_PREC_FF_RESIDUAL &&
        precision != PNJL_PREC_FP64_CERT && precision != PNJL_PREC_FP32_NEWTON)
        return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "unknown precision");
    if ((precision == PNJL_PREC_FF_RESIDUAL || precision == PNJL_PREC_FP64_CERT ||
         precision == PNJL_PREC_FP32_NEWTON) && out)
        return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "this pass gives the residual only");
    if (n == 0) return PNJL_OK;
    cudaSetDevice(ctx->device);
    const size_t nn = (size_t)n;
    size_t bytes = carve_size(5 * nn, 8) + 5 * carve_size(nn, 8) + carve_size(nn, 8) + carve_size(5 * nn, 8) +
                   carve_size(25 * nn, 8) + 5 * carve_size(nn, 8) + 4 * carve_size(3 * nn, 8);
    int rc = ensure_ws(ctx, bytes);
    if (rc) return rc;
    unsigned char *p = ctx->d_ws;
    double *dx = carve<double>(p, 5 * nn), *dT = carve<double>(p, nn), *du = carve<double>(p, nn),
           *dd = carve<double>(p, nn), *ds = carve<double>(p, nn), *dxi = carve<double>(p, nn);
    double *dom = carve<double>(p, nn), *dg = carve<double>(p, 5 * nn), *dh = carve<double>(p, 25 * nn);
    pnjl_result_soa dout{};
    dout.omega = nullptr;
    dout.pressure = carve<double>(p, nn);
    dout.rho_norm = carve<double>(p, nn);
    dout.entropy = carve<double>(p, nn);
    dout.energy = carve<double>(p, nn);
    double *dspare = carve<double>(p, nn);
    (void)dspare;
    dout.masses = carve<double>(p, 3 * nn);
    dout.rho = carve<double>(p, 3 * nn);
    dout.n_q = carve<double>(p, 3 * nn);
    dout.n_aq = carve<double>(p, 3 * nn);
    cudaStream_t s = ctx->stream;
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dx, x, 5 * nn * 8, cudaMemcpyHostToDevice, s));
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dT, T, nn * 8, cudaMemcpyHostToDevice, s));
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(du, mu_u, nn * 8, cudaMemcpyHostToDevice, s));
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dd, mu_d, nn * 8, cudaMemcpyHostToDevice, s));
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(ds, mu_s, nn * 8, cudaMemcpyHostToDevice, s));
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dxi, xi, nn * 8, cudaMemcpyHostToDevice, s));
    pnjl::EvalArgs a{};
    a.P = ctx->dp;
    a.nodes = kernel_nodes(ctx);
    const int mode = precision;  // 0 FP64, 1 FP32-Kahan, 2 float-float, 3 FP64 certification, 4 FP32 Newton
    const size_t smem = pnjl::node_smem_bytes(ctx->p_num, ctx->t_num);
    a.n = n;
    a.x = dx; a.T = dT; a.mu_u = du; a.mu_d = dd; a.mu_s = ds; a.xi = dxi;
    a.omega = dom; a.grad = dg; a.hess = dh;
    a.out = dout;
    int64_t blocks = (n + 7) / 8;
    int grid = (int)std::min<int64_t>(blocks, (int64_t)ctx->sm_count * 8);
    cudaError_t e = pnjl::launch_eval(a, mode, grid, smem, s);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "eval_kernel launch");
    ctx->stats.kernel_launches += 1;
    if (omega) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(omega, dom, nn * 8, cudaMemcpyDeviceToHost, s));
    if (grad) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(grad, dg, 5 * nn * 8, cudaMemcpyDeviceToHost, s));
    if (hess) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(hess, dh, 25 * nn * 8, cudaMemcpyDeviceToHost, s));
    if (out) {
        if (out->omega) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->omega, dom, nn * 8, cudaMemcpyDeviceToHost, s));
        if (out->pressure) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->pressure, dout.pressure, nn * 8, cudaMemcpyDeviceToHost, s));
        if (out->rho_norm) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->rho_norm, dout.rho_norm, nn * 8, cudaMemcpyDeviceToHost, s));
        if (out->entropy) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->entropy, dout.entropy, nn * 8, cudaMemcpyDeviceToHost, s));
        if (out->energy) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->energy, dout.energy, nn * 8, cudaMemcpyDeviceToHost, s));
        if (out->masses) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->masses, dout.masses, 3 * nn * 8, cudaMemcpyDeviceToHost, s));
        if (out->rho) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->rho, dout.rho, 3 * nn * 8, cudaMemcpyDeviceToHost, s));
        if (out->n_q) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->n_q, dout.n_q, 3 * nn * 8, cudaMemcpyDeviceToHost, s));
        if (out->n_aq) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->n_aq, dout.n_aq, 3 * nn * 8, cudaMemcpyDeviceToHost, s));
    }
    PNJL_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return PNJL_OK;
}

int pnjl_eval_batch(pnjl_ctx *ctx, int64_t n, const double *x, const double *T, const double *mu_u,
                    const double *mu_d, const double *mu_s, const double *xi, int32_t precision, double *omega,
                    double *grad, double *hess) {
    return eval_common(ctx, n, x, T, mu_u, mu_d, mu_s, xi, precision, omega, grad, hess, nullptr);
}

// ---- K data (build_K_data) ----------------------------------------------------------------
static int kdata_nodes(pnjl_ctx *ctx, int32_t p_num, double p_max) {
    if (ctx->d_kd_nodes && ctx->kd_p_num == p_num && ctx->kd_p_max == p_max) return PNJL_OK;
    if (!ctx->d_kd_nodes)
        PNJL_CUDA_TRY(ctx, cudaMalloc(&ctx->d_kd_nodes, 2 * (size_t)pnjl::kMaxPNodes * sizeof(double)));
    std::vector<double> pw(2 * (size_t)p_num);
    pnjl::gauss_legendre_into(p_num, 0.0, p_max, pw.data(), pw.data() + p_num);
    // the stream may still read the previous table: the copy is ordered after it
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_kd_nodes, pw.data(), pw.size() * sizeof(double), cudaMemcpyHostToDevice,
                                       ctx->stream));
    PNJL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));  // pw is released on return
    ctx->kd_p_num = p_num;
    ctx->kd_p_max = p_max;
    return PNJL_OK;
}

static int kdata_enqueue(pnjl_ctx *ctx, int64_t n, int32_t p_num, double p_max, const double *d_T,
                         const double *d_mu_u, const double *d_mu_s, const double *d_masses, const double *d_x,
                         const pnjl_kdata_soa &d_out) {
    int rc = kdata_nodes(ctx, p_num, p_max);
    if (rc) return rc;
    pnjl::KDataArgs a{};
    a.Lambda = ctx->params.Lambda;
    a.G = ctx->params.G;
    a.K = ctx->params.K;
    a.p_num = p_num;
    a.p = ctx->d_kd_nodes;
    a.w = ctx->d_kd_nodes + p_num;
    a.n = n;
    a.T = d_T; a.mu_u = d_mu_u; a.mu_s = d_mu_s; a.masses = d_masses; a.x = d_x;
    a.out = d_out;
    cudaError_t e = pnjl::launch_kdata(a, ctx->sm_count, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "kdata_kernel launch");
    ctx->stats.kernel_launches += 1;
    return PNJL_OK;
}

static int kdata_check(pnjl_ctx *ctx, int64_t n, int32_t p_num, double p_max, const double *T, const double *mu_u,
                       const double *mu_s, const double *masses, const double *x, const pnjl_kdata_soa *out) {
    if (!ctx) return PNJL_ERR_INVALID_ARGUMENT;
    if (!out) return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "null output struct");
    if (p_num < 1 || p_num > pnjl::kMaxPNodes || !(p_max > 0.0) || !std::isfinite(p_max))
        return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "p_num must be 1..512 and p_max finite and positive");
    if (n < 0 || (n > 0 && (!T || !mu_u || !mu_s || !masses || !x)))
        return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "null input array");
    return PNJL_OK;
}

int pnjl_kdata_batch_device(pnjl_ctx *ctx, int64_t n, int32_t p_num, double p_max, const double *d_T,
                            const double *d_mu_u, const double *d_mu_s, const double *d_masses, const double *d_x,
                            pnjl_kdata_soa *d_out) {
    int rc = kdata_check(ctx, n, p_num, p_max, d_T, d_mu_u, d_mu_s, d_masses, d_x, d_out);
    if (rc || n == 0) return rc;
    cudaSetDevice(ctx->device);
    return kdata_enqueue(ctx, n, p_num, p_max, d_T, d_mu_u, d_mu_s, d_masses, d_x, *d_out);
}

int pnjl_kdata_batch(pnjl_ctx *ctx, int64_t n, int32_t p_num, double p_max, const double *T, const double *mu_u,
                     const double *mu_s, const double *masses, const double *x, pnjl_kdata_soa *out) {
    int rc = kdata_check(ctx, n, p_num, p_max, T, mu_u, mu_s, masses, x, out);
    if (rc || n == 0) return rc;
    cudaSetDevice(ctx->device);
    const size_t nn = (size_t)n;
    constexpr int kFields = 17;
    double *const *hout[kFields] = {&out->A_u, &out->A_d, &out->A_s, &out->G_u, &out->G_s, &out->K0_plus,
                                    &out->K0_minus, &out->K123_plus, &out->K123_minus, &out->K4567_plus,
                                    &out->K4567_minus, &out->K8_plus, &out->K8_minus, &out->K08_plus,
                                    &out->K08_minus, &out->det_K_plus, &out->det_K_minus};
    rc = ensure_ws(ctx, (3 + kFields) * carve_size(nn, 8) + carve_size(3 * nn, 8) + carve_size(5 * nn, 8));
    if (rc) return rc;
    unsigned char *p = ctx->d_ws;
    double *dT = carve<double>(p, nn), *du = carve<double>(p, nn), *ds = carve<double>(p, nn),
           *dm = carve<double>(p, 3 * nn), *dx = carve<double>(p, 5 * nn);
    pnjl_kdata_soa dout{};
    double **dptr[kFields] = {&dout.A_u, &dout.A_d, &dout.A_s, &dout.G_u, &dout.G_s, &dout.K0_plus, &dout.K0_minus,
                              &dout.K123_plus, &dout.K123_minus, &dout.K4567_plus, &dout.K4567_minus,
                              &dout.K8_plus, &dout.K8_minus, &dout.K08_plus, &dout.K08_minus, &dout.det_K_plus,
                              &dout.det_K_minus};
    for (int k = 0; k < kFields; ++k) {
        double *d = carve<double>(p, nn);
        *dptr[k] = *hout[k] ? d : nullptr;
    }
    cudaStream_t s = ctx->stream;
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dT, T, nn * 8, cudaMemcpyHostToDevice, s));
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(du, mu_u, nn * 8, cudaMemcpyHostToDevice, s));
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(ds, mu_s, nn * 8, cudaMemcpyHostToDevice, s));
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dm, masses, 3 * nn * 8, cudaMemcpyHostToDevice, s));
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dx, x, 5 * nn * 8, cudaMemcpyHostToDevice, s));
    rc = kdata_enqueue(ctx, n, p_num, p_max, dT, du, ds, dm, dx, dout);
    if (rc) return rc;
    for (int k = 0; k < kFields; ++k)
        if (*hout[k]) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(*hout[k], *dptr[k], nn * 8, cudaMemcpyDeviceToHost, s));
    PNJL_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return PNJL_OK;
}

// ---- implicit derivatives (ThermoDerivatives.jl) -------------------------------------------
static double **deriv_field(pnjl_deriv_soa &o, int k, int &width) {
    double **f[20] = {&o.dx_dT, &o.dx_dmu, &o.dM_dT, &o.dM_dmu, &o.s, &o.n_B, &o.ds_dT, &o.ds_dmu, &o.dn_dT,
                      &o.dn_dmu, &o.pressure, &o.dP_dT, &o.dP_dmu, &o.energy, &o.deps_dT, &o.deps_dmu,
                      &o.dP_deps_n, &o.dP_dn_eps, &o.v_n_sq, &o.dmuB_dT_sigma};
    width = k < 2 ? 5 : (k < 4 ? 3 : 1);
    return f[k];
}

static int derivs_enqueue(pnjl_ctx *ctx, int64_t n, const double *d_x, const double *d_T, const double *d_mu_u,
                          const double *d_mu_d, const double *d_mu_s, const double *d_xi, const pnjl_deriv_soa &o) {
    pnjl::DerivArgs a{};
    a.P = ctx->dp;
    a.nodes = kernel_nodes(ctx);
    a.n = n;
    a.x = d_x; a.T = d_T; a.mu_u = d_mu_u; a.mu_d = d_mu_d; a.mu_s = d_mu_s; a.xi = d_xi;
    a.out = o;
    const size_t smem = pnjl::node_smem_bytes(ctx->p_num, ctx->t_num);
    const int64_t blocks = (n + 7) / 8;
    const int grid = (int)std::min<int64_t>(blocks, (int64_t)ctx->sm_count * 8);
    cudaError_t e = pnjl::launch_deriv(a, grid, smem, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "deriv_kernel launch");
    ctx->stats.kernel_launches += 1;
    return PNJL_OK;
}

static int derivs_check(pnjl_ctx *ctx, int64_t n, const double *x, const double *T, const double *mu_u,
                        const double *mu_d, const double *mu_s, const double *xi, const pnjl_deriv_soa *out) {
    if (!ctx) return PNJL_ERR_INVALID_ARGUMENT;
    if (ctx->p_num == 0) return fail(ctx, PNJL_ERR_NO_NODES, "call pnjl_set_nodes first");
    if (!out) return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "null output struct");
    if (n < 0 || (n > 0 && (!x || !T || !mu_u || !mu_d || !mu_s || !xi)))
        return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "null input array");
    return PNJL_OK;
}

int pnjl_derivs_batch_device(pnjl_ctx *ctx, int64_t n, const double *d_x, const double *d_T, const double *d_mu_u,
                             const double *d_mu_d, const double *d_mu_s, const double *d_xi, pnjl_deriv_soa *d_out) {
    int rc = derivs_check(ctx, n, d_x, d_T, d_mu_u, d_mu_d, d_mu_s, d_xi, d_out);
    if (rc || n == 0) return rc;
    cudaSetDevice(ctx->device);
    return derivs_enqueue(ctx, n, d_x, d_T, d_mu_u, d_mu_d, d_mu_s, d_xi, *d_out);
}

int pnjl_derivs_batch(pnjl_ctx *ctx, int64_t n, const double *x, const double *T, const double *mu_u,
                      const double *mu_d, const double *mu_s, const double *xi, pnjl_deriv_soa *out) {
    int rc = derivs_check(ctx, n, x, T, mu_u, mu_d, mu_s, xi, out);
    if (rc || n == 0) return rc;
    cudaSetDevice(ctx->device);
    const size_t nn = (size_t)n;
    rc = ensure_ws(ctx, carve_size(5 * nn, 8) + 5 * carve_size(nn, 8) + 4 * carve_size(5 * nn, 8) +
                            18 * carve_size(nn, 8));
    if (rc) return rc;
    unsigned char *p = ctx->d_ws;
    double *dx = carve<double>(p, 5 * nn), *dT = carve<double>(p, nn), *du = carve<double>(p, nn),
           *dd = carve<double>(p, nn), *ds = carve<double>(p, nn), *dxi = carve<double>(p, nn);
    pnjl_deriv_soa dout{};
    pnjl_deriv_soa hout = *out;
    for (int k = 0; k < 20; ++k) {
        int w = 1;
        double **h = deriv_field(hout, k, w);
        double **d = deriv_field(dout, k, w);
        double *buf = carve<double>(p, (size_t)w * nn);
        *d = *h ? buf : nullptr;
    }
    cudaStream_t s = ctx->stream;
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dx, x, 5 * nn * 8, cudaMemcpyHostToDevice, s));
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dT, T, nn * 8, cudaMemcpyHostToDevice, s));
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(du, mu_u, nn * 8, cudaMemcpyHostToDevice, s));
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dd, mu_d, nn * 8, cudaMemcpyHostToDevice, s));
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(ds, mu_s, nn * 8, cudaMemcpyHostToDevice, s));
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dxi, xi, nn * 8, cudaMemcpyHostToDevice, s));
    rc = derivs_enqueue(ctx, n, dx, dT, du, dd, ds, dxi, dout);
    if (rc) return rc;
    for (int k = 0; k < 20; ++k) {
        int w = 1;
        double **h = deriv_field(hout, k, w);
        double **d = deriv_field(dout, k, w);
        if (*h) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(*h, *d, (size_t)w * nn * 8, cudaMemcpyDeviceToHost, s));
    }
    PNJL_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return PNJL_OK;
}

int pnjl_thermo_batch(pnjl_ctx *ctx, int64_t n, const double *x, const double *T, const double *mu_u,
                      const double *mu_d, const double *mu_s, const double *xi, pnjl_result_soa *out) {
    return eval_common(ctx, n, x, T, mu_u, mu_d, mu_s, xi, PNJL_PREC_FP64, nullptr, nullptr, nullptr, out);
}

// Chunks of the mixed per-point pipeline for n points: the tuned value, or automatic -- one
// chunk per ~2 points for every resident warp (sm_count x 16 warps x 2), at most 4.
static int pipeline_chunks(const pnjl_ctx *ctx, int64_t n) {
    int C = ctx->pipeline_chunks;
    if (C < 0) return -1;  // the two kernels one after the other
    if (C == 0) return 1;  // automatic: the fused kernel
    C = std::min<int>(C, pnjl::kMaxPipelineChunks);
    return (int)std::max<int64_t>(1, std::min<int64_t>(C, n / 64 > 0 ? n / 64 : 1));
}

// The arguments of the mixed solve restricted to points [lo, hi): inputs, per-point seeds,
// outputs and every per-slot scratch array offset by lo (slots are chunk-local point
// indices), and the chunk's own queue heads and list length in the control block.
static pnjl::SolveArgs chunk_args(const pnjl::SolveArgs &a, int64_t lo, int64_t hi, long long *ctrl3) {
    pnjl::SolveArgs c = a;
    const int S = a.n_seeds;
    c.n = hi - lo;
    c.T = a.T + lo; c.mu_u = a.mu_u + lo; c.mu_d = a.mu_d + lo; c.mu_s = a.mu_s + lo; c.xi = a.xi + lo;
    if (a.point_seeds) c.point_seeds = a.point_seeds + 5 * lo;
    auto sh = [lo](auto *p, int64_t k) { return p ? p + k * lo : p; };
    c.out.x = sh(a.out.x, 5);
    c.out.omega = sh(a.out.omega, 1);
    c.out.pressure = sh(a.out.pressure, 1);
    c.out.rho_norm = sh(a.out.rho_norm, 1);
    c.out.entropy = sh(a.out.entropy, 1);
    c.out.energy = sh(a.out.energy, 1);
    c.out.masses = sh(a.out.masses, 3);
    c.out.rho = sh(a.out.rho, 3);
    c.out.n_q = sh(a.out.n_q, 3);
    c.out.n_aq = sh(a.out.n_aq, 3);
    c.out.residual_norm = sh(a.out.residual_norm, 1);
    c.out.iterations = sh(a.out.iterations, 1);
    c.out.chosen_seed = sh(a.out.chosen_seed, 1);
    c.out.status = sh(a.out.status, 1);
    c.out.converged = sh(a.out.converged, 1);
    c.cand = sh(a.cand, S + 1);
    c.done = sh(a.done, 1);
    c.roots = sh(a.roots, 5 * S);
    c.root_flag = sh(a.root_flag, S);
    c.anchor_state = sh(a.anchor_state, 1);
    c.anchor_omega = sh(a.anchor_omega, 1);
    c.list = sh(a.list, 1);
    c.list_mode = sh(a.list_mode, 1);
    c.queue = ctrl3;
    c.list_count = ctrl3 + 1;
    c.queue2 = ctrl3 + 2;
    c.points_done = nullptr;
    c.cert_warps = 0;
    c.jobs = nullptr;
    c.job_ready = nullptr;
    c.job_count = c.job_head = nullptr;
    return c;
}

// Device-side resources one batched solve writes to: the context's own, or a plan segment's.
struct SolveRes {
    long long *ctrl;               // kCtrlSlots counters and queue heads (zeroed by the enqueue)
    unsigned char *scratch;        // at least solve_scratch_bytes(n, opts)
    const double *seed_tables;     // device copy of the seed tables (cold | hot, 16 rows each)
    const unsigned char *vmap;     // device copy of the verification map, or null
    cudaStream_t s, s2;            // s2: second stream of the chunk pipeline
    const cudaEvent_t *ev_chunk;   // kMaxPipelineChunks events (no timing)
    cudaEvent_t ev_join;
    cudaEvent_t ev_mid;            // optional: end of the first kernel (timed split) ...
    long long *ctrl_snap;          // ... and the counters at that moment
};

static size_t al256(size_t b) { return (b + 255) & ~size_t(255); }

// Scratch bytes of one batched solve of n points.
static size_t solve_scratch_bytes(int64_t n, const pnjl_solve_opts *o) {
    const bool mixed = o->precision == PNJL_PREC_MIXED;
    const int S = (o->n_seeds > 0 && o->seed_table) ? o->n_seeds : 0;
    const size_t nn = (size_t)n;
    if (o->seed_mode == PNJL_SEEDS_TABLE && !mixed)
        return al256(nn * sizeof(int)) + nn * o->n_seeds * sizeof(pnjl::CandRec);
    if (mixed && S > 0)
        return al256(nn * sizeof(int)) + al256(nn * S * sizeof(int)) + al256(nn * sizeof(int)) +
               al256(nn * (S + 1) * sizeof(int)) + al256(nn * sizeof(int)) +
               al256(nn * (S + 1) * sizeof(pnjl::CandRec)) + al256(nn * S * 5 * sizeof(double)) +
               al256(nn * sizeof(long long)) + al256(nn * sizeof(double)) +
               al256(nn * (S + 1) * sizeof(pnjl::CertJob));
    return 0;
}

// Enqueue one batched solve (memsets and kernels only: no host copies, no allocation, no
// host synchronisation -- so it can also be captured into a CUDA graph).  `launches` receives
// the kernel count; `split` whether ev_mid / ctrl_snap were recorded.
static cudaError_t solve_enqueue(const pnjl_ctx *ctx, const pnjl::KernelNodes &nodes, int64_t n, const double *d_T,
                                 const double *d_mu_u, const double *d_mu_d, const double *d_mu_s, const double *d_xi,
                                 const pnjl_solve_opts *opts, const pnjl_result_soa &d_out, const SolveRes &r,
                                 int *launches, bool *split) {
    cudaStream_t s = r.s;
    const bool has_table = opts->n_seeds > 0 && opts->seed_table;
    pnjl::SolveArgs a{};
    const bool mixed = opts->precision == PNJL_PREC_MIXED;
    const int S = has_table ? opts->n_seeds : 0;
    cudaError_t e = cudaSuccess;
    if (opts->seed_mode == PNJL_SEEDS_TABLE && !mixed) {
        const size_t cnt = al256((size_t)n * sizeof(int));
        a.done = (int *)r.scratch;
        a.cand = (pnjl::CandRec *)(r.scratch + cnt);
        if ((e = cudaMemsetAsync(a.done, 0, (size_t)n * sizeof(int), s)) != cudaSuccess) return e;
    } else if (mixed && S > 0) {
        // slots: every point (table mode) or the points the per-point kernel defers
        const size_t nn = (size_t)n;
        const size_t b_done = al256(nn * sizeof(int)), b_flag = al256(nn * S * sizeof(int));
        const size_t b_mode = al256(nn * sizeof(int)), b_ready = al256(nn * (S + 1) * sizeof(int));
        const size_t b_anchor = al256(nn * sizeof(int));
        const size_t b_cand = al256(nn * (S + 1) * sizeof(pnjl::CandRec)), b_roots = al256(nn * S * 5 * sizeof(double));
        const size_t b_list = al256(nn * sizeof(long long));
        unsigned char *q = r.scratch;
        a.done = (int *)q;
        q += b_done;
        a.root_flag = (int *)q;
        q += b_flag;
        a.list_mode = (int *)q;
        q += b_mode;
        a.job_ready = (int *)q;
        q += b_ready;
        a.anchor_state = (int *)q;
        q += b_anchor;
        a.cand = (pnjl::CandRec *)q;
        q += b_cand;
        a.roots = (double *)q;
        q += b_roots;
        a.list = (long long *)q;
        q += b_list;
        a.anchor_omega = (double *)q;
        q += al256(nn * sizeof(double));
        a.jobs = (pnjl::CertJob *)q;
        // done, root_flag, list_mode, job_ready and anchor_state are adjacent: one memset clears them
        if ((e = cudaMemsetAsync(r.scratch, 0, b_done + b_flag + b_mode + b_ready + b_anchor, s)) != cudaSuccess)
            return e;
    }
    if ((e = cudaMemsetAsync(r.ctrl, 0, pnjl::kCtrlSlots * sizeof(long long), s)) != cudaSuccess) return e;
    a.P = ctx->dp;
    a.nodes = nodes;
    const size_t smem = pnjl::node_smem_bytes(nodes.p_num, nodes.t_num);
    a.n = n;
    a.T = d_T; a.mu_u = d_mu_u; a.mu_d = d_mu_d; a.mu_s = d_mu_s; a.xi = d_xi;
    a.seed_mode = opts->seed_mode;
    a.n_seeds = S;
    a.seed_table = r.seed_tables;
    a.seed_table_hot = (has_table && opts->seed_table_hot) ? r.seed_tables + 80 : nullptr;
    a.hot_T_MeV = opts->hot_T_MeV;
    a.point_seeds = opts->point_seeds;
    pnjl::fill_solve_opts(opts, a.opts);
    a.opts.ready_polls = ctx->ready_polls;
    a.opts.verdict_polls = ctx->verdict_polls;
    if (pnjl::verify_map_cells(opts)) a.opts.vmap = r.vmap;
    a.out = d_out;
    a.queue = r.ctrl;
    a.stats = r.ctrl + 1;
    a.list_count = r.ctrl + 1 + pnjl::kStatCount;
    a.queue2 = r.ctrl + 2 + pnjl::kStatCount;
    a.points_done = r.ctrl + 3 + pnjl::kStatCount;
    a.job_count = r.ctrl + 4 + pnjl::kStatCount;
    a.job_head = r.ctrl + 5 + pnjl::kStatCount;
    a.cert_warps = 0;
    const int group = ctx->group;
    int grid = 0, grid_tasks = 0, grid_fused = 0;
    *launches = 1;
    if (mixed) {
        const int64_t wpb = pnjl::kSolveThreads / 32;
        auto occ_of = [&](int kernel) {
            int occ = pnjl::solve_mixed_occupancy(kernel, smem);
            if (occ < 1) occ = 1;
            if (ctx->blocks_per_sm > 0 && ctx->blocks_per_sm < occ) occ = ctx->blocks_per_sm;
            return (int64_t)occ;
        };
        const bool table = opts->seed_mode == PNJL_SEEDS_TABLE;
        grid = (int)std::min<int64_t>((int64_t)ctx->sm_count * occ_of(pnjl::kMixedPoints), (n + wpb - 1) / wpb);
        const int64_t task_need = table ? (n * S + wpb - 1) / wpb : (int64_t)ctx->sm_count * occ_of(pnjl::kMixedTasks);
        grid_tasks = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx->sm_count * occ_of(pnjl::kMixedTasks),
                                                                 task_need));
        const int64_t wpf = pnjl::kFusedThreads / 32;
        grid_fused = (int)std::max<int64_t>(
            1, std::min<int64_t>((int64_t)ctx->sm_count * occ_of(pnjl::kMixedFused), (n * (S + 1) + wpf - 1) / wpf));
        *launches = table ? 1 : (S > 0 ? 2 : 1);
    } else {
        const int64_t n_tasks = opts->seed_mode == PNJL_SEEDS_TABLE ? n * (int64_t)opts->n_seeds : n;
        grid = grid_for(ctx, group, smem, n_tasks);
    }
    *split = false;
    const bool two = mixed && *launches == 2;
    if (!mixed) {
        e = pnjl::launch_solve(a, group, grid, smem, s);
    } else if (opts->seed_mode == PNJL_SEEDS_TABLE) {
        e = pnjl::launch_mixed_tasks(a, grid_tasks, smem, s);
    } else if (two && pipeline_chunks(ctx, n) == 1) {
        // one launch: the per-point seeds and the tasks they defer (verification, MultiSeed
        // fallback) share the persistent grid; the first cert_warps warps of each block certify
        a.cert_warps = ctx->cert_warps;
        e = pnjl::launch_mixed_fused(a, grid_fused, smem, s);
        *launches = 1;
    } else if (two && pipeline_chunks(ctx, n) > 1) {
        // chunk pipeline: the per-point kernel of chunk c+1 (stream s) runs while the task
        // kernel of chunk c (stream s2) works through the points chunk c deferred; each fills
        // the other's tail.  The chunks' queue heads and list lengths are separate slots.
        const int C = pipeline_chunks(ctx, n);
        for (int c = 0; c < C && e == cudaSuccess; ++c) {
            const int64_t lo = n * c / C, hi = n * (c + 1) / C;
            const pnjl::SolveArgs ac = chunk_args(a, lo, hi, r.ctrl + pnjl::kChunkCtrlBase + 3 * c);
            const int g1 = (int)std::max<int64_t>(1, std::min<int64_t>(grid, (hi - lo + 7) / 8));
            if ((e = pnjl::launch_mixed_points(ac, g1, smem, s)) != cudaSuccess) break;
            if ((e = cudaEventRecord(r.ev_chunk[c], s)) != cudaSuccess) break;
            if ((e = cudaStreamWaitEvent(r.s2, r.ev_chunk[c], 0)) != cudaSuccess) break;
            e = pnjl::launch_mixed_tasks(ac, grid_tasks, smem, r.s2);
        }
        if (e == cudaSuccess && (e = cudaEventRecord(r.ev_join, r.s2)) == cudaSuccess)
            e = cudaStreamWaitEvent(s, r.ev_join, 0);
        *launches = 2 * C;
    } else {
        e = pnjl::launch_mixed_points(a, grid, smem, s);
        if (e == cudaSuccess && two) {
            if (r.ev_mid && r.ctrl_snap) {
                // the per-point kernel's own time and counters, then the task kernel
                if ((e = cudaEventRecord(r.ev_mid, s)) != cudaSuccess) return e;
                if ((e = cudaMemcpyAsync(r.ctrl_snap, r.ctrl, pnjl::kCtrlSlots * sizeof(long long),
                                         cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
                    return e;
                *split = true;
            }
            e = pnjl::launch_mixed_tasks(a, grid_tasks, smem, s);
        }
    }
    return e;
}

int pnjl_solve_batch_device(pnjl_ctx *ctx, int64_t n, const double *d_T, const double *d_mu_u, const double *d_mu_d,
                            const double *d_mu_s, const double *d_xi, const pnjl_solve_opts *opts,
                            pnjl_result_soa *d_out) {
    if (!ctx) return PNJL_ERR_INVALID_ARGUMENT;
    if (ctx->p_num == 0) return fail(ctx, PNJL_ERR_NO_NODES, "call pnjl_set_nodes first");
    int rc = check_opts(ctx, opts);
    if (rc) return rc;
    if (n < 0 || !d_out || (n > 0 && (!d_T || !d_mu_u || !d_mu_d || !d_mu_s || !d_xi)))
        return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "null array");
    if (n == 0) return PNJL_OK;
    cudaSetDevice(ctx->device);
    cudaStream_t s = ctx->stream;
    if (opts->n_seeds > 0 && opts->seed_table) {
        PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_seed_tables, opts->seed_table, opts->n_seeds * 5 * sizeof(double),
                                           cudaMemcpyHostToDevice, s));
        if (opts->seed_table_hot)
            PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_seed_tables + 80, opts->seed_table_hot,
                                               opts->n_seeds * 5 * sizeof(double), cudaMemcpyHostToDevice, s));
    }
    if (const int64_t cells = pnjl::verify_map_cells(opts)) {
        if ((size_t)cells > ctx->vmap_cap) {
            PNJL_CUDA_TRY(ctx, cudaStreamSynchronize(s));
            cudaFree(ctx->d_vmap);
            ctx->d_vmap = nullptr;
            ctx->vmap_cap = 0;
            if (cudaMalloc(&ctx->d_vmap, (size_t)cells) != cudaSuccess)
                return fail(ctx, PNJL_ERR_OUT_OF_MEMORY, "verification map allocation failed");
            ctx->vmap_cap = (size_t)cells;
        }
        PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_vmap, opts->verify_map, (size_t)cells, cudaMemcpyHostToDevice, s));
    }
    if (const size_t bytes = solve_scratch_bytes(n, opts)) {
        rc = ensure_scratch(ctx, bytes);
        if (rc) return rc;
    }
    SolveRes r{ctx->d_ctrl, ctx->d_scratch, ctx->d_seed_tables, ctx->d_vmap, s, ctx->stream2, ctx->ev_chunk,
               ctx->ev_join, ctx->ev_mid, ctx->d_ctrl_snap};
    PNJL_CUDA_TRY(ctx, cudaEventRecord(ctx->ev0, s));
    int launches = 0;
    bool split = false;
    const cudaError_t e = solve_enqueue(ctx, kernel_nodes(ctx), n, d_T, d_mu_u, d_mu_d, d_mu_s, d_xi, opts, *d_out,
                                        r, &launches, &split);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "solve kernel launch");
    ctx->split_last = split;
    PNJL_CUDA_TRY(ctx, cudaEventRecord(ctx->ev1, s));
    ctx->stats.kernel_launches += launches;
    ctx->stats.points = n;
    return PNJL_OK;
}


int pnjl_mlp_param_count(void) { return pnjl::kParamCount; }

int pnjl_mlp_init(pnjl_ctx *ctx, uint64_t seed) {
    if (!ctx) return PNJL_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    auto &M = ctx->mlp;
    if (!M.params) {
        PNJL_CUDA_TRY(ctx, cudaMalloc(&M.params, 4 * (size_t)pnjl::kParamCount * sizeof(float)));
        PNJL_CUDA_TRY(ctx, cudaMalloc(&M.wb, (size_t)pnjl::kParamCount * sizeof(__nv_bfloat16)));
        PNJL_CUDA_TRY(ctx, cudaMalloc(&M.step, sizeof(long long)));
        PNJL_CUDA_TRY(ctx, cudaMalloc(&M.loss, sizeof(float)));
        PNJL_CUDA_TRY(ctx, cudaMalloc(&M.partial, (size_t)pnjl::kMaxGradSlots * (pnjl::kParamCount + 1) * sizeof(float)));
        PNJL_CUDA_TRY(ctx, pnjl::mlp_setup_attributes());
    }
    // Kaiming-uniform weights (bound sqrt(6 / fan_in)), zero biases
    const int H = pnjl::mlp::H, IN = pnjl::mlp::IN, OUT = pnjl::mlp::OUT;
    std::vector<float> w(pnjl::kParamCount, 0.0f);
    uint64_t s = seed;
    auto fill = [&](int off, int rows, int cols) {
        const double bound = std::sqrt(6.0 / cols);
        for (int i = 0; i < rows * cols; ++i) w[off + i] = (float)((2.0 * uniform01(s) - 1.0) * bound);
    };
    int off = 0;
    fill(off, H, IN); off += H * IN + H;
    fill(off, H, H); off += H * H + H;
    fill(off, H, H); off += H * H + H;
    fill(off, OUT, H);
    for (int i = 0; i < OUT * H; ++i) w[off + i] *= 0.1f;  // small output layer
    PNJL_CUDA_TRY(ctx, cudaMemcpy(M.params, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice));
    PNJL_CUDA_TRY(ctx, cudaMemset(M.params + pnjl::kParamCount, 0, 3 * (size_t)pnjl::kParamCount * sizeof(float)));
    PNJL_CUDA_TRY(ctx, cudaMemset(M.step, 0, sizeof(long long)));
    PNJL_CUDA_TRY(ctx, pnjl::mlp_refresh_bf16(mlp_dev(ctx), ctx->stream));
    PNJL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    M.ready = true;
    M.trained = false;
    return PNJL_OK;
}

int pnjl_mlp_set_scaling(pnjl_ctx *ctx, const double *in_shift, const double *in_scale, const double *out_shift,
                         const double *out_scale) {
    if (!ctx || !in_shift || !in_scale || !out_shift || !out_scale) return PNJL_ERR_INVALID_ARGUMENT;
    auto &sc = ctx->mlp.sc;
    for (int k = 0; k < 3; ++k) {
        if (!(in_scale[k] != 0.0) || !std::isfinite(in_scale[k]) || !std::isfinite(in_shift[k]))
            return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "input scaling must be finite and non-zero");
        sc.in_shift[k] = in_shift[k];
        sc.in_scale[k] = in_scale[k];
    }
    for (int k = 0; k < 5; ++k) {
        if (!(out_scale[k] != 0.0) || !std::isfinite(out_scale[k]) || !std::isfinite(out_shift[k]))
            return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "output scaling must be finite and non-zero");
        sc.out_shift[k] = out_shift[k];
        sc.out_scale[k] = out_scale[k];
    }
    ctx->mlp.scaled = true;
    return PNJL_OK;
}

static int mlp_upload(pnjl_ctx *ctx, int64_t n, const double *T, const double *mu, const double *xi,
                      const double *targets) {
    int rc = mlp_ensure_data(ctx, (size_t)n);
    if (rc) return rc;
    const size_t nn = (size_t)n;
    rc = ensure_ws(ctx, 8 * nn * sizeof(double) + 1024);
    if (rc) return rc;
    double *dT = (double *)ctx->d_ws, *dmu = dT + nn, *dxi = dmu + nn, *dt = dxi + nn;
    cudaStream_t s = ctx->stream;
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dT, T, nn * 8, cudaMemcpyHostToDevice, s));
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dmu, mu, nn * 8, cudaMemcpyHostToDevice, s));
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dxi, xi, nn * 8, cudaMemcpyHostToDevice, s));
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dt, targets, 5 * nn * 8, cudaMemcpyHostToDevice, s));
    PNJL_CUDA_TRY(ctx, pnjl::mlp_prepare(ctx->mlp.sc, n, dT, dmu, dxi, dt, ctx->mlp.x, ctx->mlp.y, s));
    return PNJL_OK;
}

int pnjl_mlp_loss_grad(pnjl_ctx *ctx, int64_t n, const double *T, const double *mu, const double *xi,
                       const double *targets, double *loss, float *grad) {
    if (!ctx) return PNJL_ERR_INVALID_ARGUMENT;
    int rc = mlp_require(ctx, true);
    if (rc) return rc;
    if (n <= 0 || n > (1 << 24) || !T || !mu || !xi || !targets) return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "bad batch");
    cudaSetDevice(ctx->device);
    rc = mlp_upload(ctx, n, T, mu, xi, targets);
    if (rc) return rc;
    pnjl::TrainBatch b{ctx->mlp.x, ctx->mlp.y, nullptr, n, (int)n, 0, ctx->mlp.step, ctx->mlp.loss};
    pnjl::AdamCfg c{};
    PNJL_CUDA_TRY(ctx, pnjl::mlp_launch_step(mlp_dev(ctx), b, c, false, ctx->stream));
    float l = 0.f;
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(&l, ctx->mlp.loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    if (grad)
        PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(grad, ctx->mlp.params + pnjl::kParamCount, pnjl::kParamCount * sizeof(float),
                                           cudaMemcpyDeviceToHost, ctx->stream));
    PNJL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (loss) *loss = l;
    ctx->stats.kernel_launches += 3;
    return PNJL_OK;
}

int pnjl_mlp_train(pnjl_ctx *ctx, int64_t n, const double *T, const double *mu, const double *xi,
                   const double *targets, int32_t epochs, int32_t batch, double lr, uint64_t shuffle_seed,
                   double *last_loss) {
    if (!ctx) return PNJL_ERR_INVALID_ARGUMENT;
    int rc = mlp_require(ctx, true);
    if (rc) return rc;
    if (n <= 0 || n > INT32_MAX || epochs < 1 || batch < 32 || batch % 32 || !(lr > 0) || !T || !mu || !xi ||
        !targets)
        return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "bad training arguments (batch: multiple of 32)");
    cudaSetDevice(ctx->device);
    rc = mlp_upload(ctx, n, T, mu, xi, targets);
    if (rc) return rc;
    rc = mlp_ensure_perm(ctx, (size_t)n * (size_t)epochs);
    if (rc) return rc;
    cudaStream_t s = ctx->stream;
    const long long spe = (n + batch - 1) / batch;
    pnjl::TrainBatch b{ctx->mlp.x, ctx->mlp.y, ctx->mlp.perm, n, batch, spe, ctx->mlp.step, ctx->mlp.loss};
    pnjl::AdamCfg c{lr, lr * 0.01, 0.9f, 0.999f, 1e-8f, spe * (long long)epochs};
    PNJL_CUDA_TRY(ctx, cudaMemsetAsync(ctx->mlp.params + 2 * pnjl::kParamCount, 0,
                                       2 * (size_t)pnjl::kParamCount * sizeof(float), s));
    PNJL_CUDA_TRY(ctx, cudaMemsetAsync(ctx->mlp.step, 0, sizeof(long long), s));
    // every epoch's shuffle (Fisher-Yates on a splitmix64 stream), uploaded once
    std::vector<int> perm((size_t)n * (size_t)epochs);
    uint64_t rs = shuffle_seed;
    for (int ep = 0; ep < epochs; ++ep) {
        int *p = perm.data() + (size_t)ep * (size_t)n;
        for (long long i = 0; i < n; ++i) p[i] = (int)i;
        for (long long i = n - 1; i > 0; --i) {
            const long long j = (long long)(splitmix64(rs) % (uint64_t)(i + 1));
            std::swap(p[i], p[j]);
        }
    }
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->mlp.perm, perm.data(), perm.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    // one epoch of training steps as a CUDA graph, replayed once per epoch
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    PNJL_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    PNJL_CUDA_TRY(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaError_t ce = cudaSuccess;
    for (long long k = 0; k < spe && ce == cudaSuccess; ++k) ce = pnjl::mlp_launch_step(mlp_dev(ctx), b, c, true, s);
    cudaError_t ee = cudaStreamEndCapture(s, &graph);
    if (ce != cudaSuccess || ee != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return cuda_fail(ctx, ce != cudaSuccess ? ce : ee, "MLP epoch capture");
    }
    ce = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return cuda_fail(ctx, ce, "MLP graph instantiate");
    float l = 0.f;
    for (int ep = 0; ep < epochs && ce == cudaSuccess; ++ep) ce = cudaGraphLaunch(exec, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce == cudaSuccess) ce = cudaMemcpy(&l, ctx->mlp.loss, sizeof(float), cudaMemcpyDeviceToHost);
    cudaGraphExecDestroy(exec);
    if (ce != cudaSuccess) return cuda_fail(ctx, ce, "MLP training");
    ctx->stats.kernel_launches += 3 * spe * (long long)epochs;
    if (last_loss) *last_loss = l;
    ctx->mlp.trained = true;
    return PNJL_OK;
}

int pnjl_mlp_infer_device(pnjl_ctx *ctx, int64_t n, const double *d_T, const double *d_mu, const double *d_xi,
                          double *d_seeds) {
    if (!ctx) return PNJL_ERR_INVALID_ARGUMENT;
    int rc = mlp_require(ctx, true);
    if (rc) return rc;
    if (n < 0 || (n > 0 && (!d_T || !d_mu || !d_xi || !d_seeds))) return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "null array");
    if (n == 0) return PNJL_OK;
    cudaSetDevice(ctx->device);
    PNJL_CUDA_TRY(ctx, pnjl::mlp_launch_infer(mlp_dev(ctx), ctx->mlp.sc, n, d_T, d_mu, d_xi, d_seeds, ctx->sm_count,
                                              ctx->stream));
    ctx->stats.kernel_launches += 1;
    return PNJL_OK;
}

int pnjl_mlp_infer(pnjl_ctx *ctx, int64_t n, const double *T, const double *mu, const double *xi, double *seeds) {
    if (!ctx) return PNJL_ERR_INVALID_ARGUMENT;
    int rc = mlp_require(ctx, true);
    if (rc) return rc;
    if (n < 0 || (n > 0 && (!T || !mu || !xi || !seeds))) return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "null array");
    if (n == 0) return PNJL_OK;
    cudaSetDevice(ctx->device);
    const size_t nn = (size_t)n;
    rc = ensure_ws(ctx, 8 * nn * sizeof(double) + 1024);
    if (rc) return rc;
    double *dT = (double *)ctx->d_ws, *dmu = dT + nn, *dxi = dmu + nn, *ds = dxi + nn;
    cudaStream_t s = ctx->stream;
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dT, T, nn * 8, cudaMemcpyHostToDevice, s));
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dmu, mu, nn * 8, cudaMemcpyHostToDevice, s));
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dxi, xi, nn * 8, cudaMemcpyHostToDevice, s));
    rc = pnjl_mlp_infer_device(ctx, n, dT, dmu, dxi, ds);
    if (rc) return rc;
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(seeds, ds, 5 * nn * 8, cudaMemcpyDeviceToHost, s));
    PNJL_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return PNJL_OK;
}

int pnjl_mlp_get_params(pnjl_ctx *ctx, float *out, int64_t count) {
    if (!ctx || !out || count != pnjl::kParamCount) return PNJL_ERR_INVALID_ARGUMENT;
    int rc = mlp_require(ctx, false);
    if (rc) return rc;
    PNJL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    PNJL_CUDA_TRY(ctx, cudaMemcpy(out, ctx->mlp.params, count * sizeof(float), cudaMemcpyDeviceToHost));
    return PNJL_OK;
}

int pnjl_mlp_set_params(pnjl_ctx *ctx, const float *in, int64_t count) {
    if (!ctx || !in || count != pnjl::kParamCount) return PNJL_ERR_INVALID_ARGUMENT;
    int rc = mlp_require(ctx, false);
    if (rc) return rc;
    PNJL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    PNJL_CUDA_TRY(ctx, cudaMemcpy(ctx->mlp.params, in, count * sizeof(float), cudaMemcpyHostToDevice));
    PNJL_CUDA_TRY(ctx, pnjl::mlp_refresh_bf16(mlp_dev(ctx), ctx->stream));
    PNJL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->mlp.trained = true;
    return PNJL_OK;
}

int pnjl_solve_batch_learned_device(pnjl_ctx *ctx, int64_t n, const double *d_T, const double *d_mu_u,
                                    const double *d_mu_d, const double *d_mu_s, const double *d_xi,
                                    const pnjl_solve_opts *opts, pnjl_result_soa *d_out) {
    if (!ctx || !opts) return PNJL_ERR_INVALID_ARGUMENT;
    int rc = mlp_require(ctx, true);
    if (rc) return rc;
    if (n <= 0) return n == 0 ? PNJL_OK : fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "n < 0");
    cudaSetDevice(ctx->device);
    auto &M = ctx->mlp;
    const size_t need = (size_t)n * 5;
    if (need > M.seeds_cap) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(M.seeds);
        M.seeds = nullptr;
        M.seeds_cap = 0;
        if (cudaMalloc(&M.seeds, need * sizeof(double)) != cudaSuccess)
            return fail(ctx, PNJL_ERR_OUT_OF_MEMORY, "seed buffer allocation failed");
        M.seeds_cap = need;
    }
    rc = pnjl_mlp_infer_device(ctx, n, d_T, d_mu_u, d_xi, M.seeds);
    if (rc) return rc;
    pnjl_solve_opts o = *opts;
    o.seed_mode = PNJL_SEEDS_PER_POINT;
    o.point_seeds = M.seeds;
    return pnjl_solve_batch_device(ctx, n, d_T, d_mu_u, d_mu_d, d_mu_s, d_xi, &o, d_out);
}

// Host-pointer solve: inputs to the workspace, the device solve (multi-seed/per-point, or
// learned-seed), results back; synchronous.
static int solve_batch_host(pnjl_ctx *ctx, int64_t n, const double *T, const double *mu_u, const double *mu_d,
                            const double *mu_s, const double *xi, const pnjl_solve_opts *opts, pnjl_result_soa *out,
                            bool learned) {
    if (!ctx) return PNJL_ERR_INVALID_ARGUMENT;
    if (ctx->p_num == 0) return fail(ctx, PNJL_ERR_NO_NODES, "call pnjl_set_nodes first");
    int rc = check_opts(ctx, opts);
    if (rc) return rc;
    if (learned) {
        rc = mlp_require(ctx, true);
        if (rc) return rc;
    }
    if (n < 0 || !out || (n > 0 && (!T || !mu_u || !mu_d || !mu_s || !xi)))
        return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "null array");
    if (n == 0) return PNJL_OK;
    cudaSetDevice(ctx->device);
    const size_t nn = (size_t)n;
    const bool per_point = !learned && opts->seed_mode == PNJL_SEEDS_PER_POINT;
    size_t bytes = 5 * carve_size(nn, 8) + (per_point ? carve_size(5 * nn, 8) : 0) + carve_size(5 * nn, 8) +
                   6 * carve_size(nn, 8) + 4 * carve_size(3 * nn, 8) + 3 * carve_size(nn, 4) + carve_size(nn, 1);
    rc = ensure_ws(ctx, bytes);
    if (rc) return rc;
    unsigned char *p = ctx->d_ws;
    double *dT = carve<double>(p, nn), *du = carve<double>(p, nn), *dd = carve<double>(p, nn),
           *ds = carve<double>(p, nn), *dxi = carve<double>(p, nn);
    double *dseeds = per_point ? carve<double>(p, 5 * nn) : nullptr;
    pnjl_result_soa d{};
    d.x = carve<double>(p, 5 * nn);
    d.omega = carve<double>(p, nn);
    d.pressure = carve<double>(p, nn);
    d.rho_norm = carve<double>(p, nn);
    d.entropy = carve<double>(p, nn);
    d.energy = carve<double>(p, nn);
    d.residual_norm = carve<double>(p, nn);
    d.masses = carve<double>(p, 3 * nn);
    d.rho = carve<double>(p, 3 * nn);
    d.n_q = carve<double>(p, 3 * nn);
    d.n_aq = carve<double>(p, 3 * nn);
    d.iterations = carve<int32_t>(p, nn);
    d.chosen_seed = carve<int32_t>(p, nn);
    d.status = carve<int32_t>(p, nn);
    d.converged = carve<uint8_t>(p, nn);
    cudaStream_t s = ctx->stream;
    // inputs and outputs cross through a pinned mirror of the workspace: one DMA each way
    // (the CUDA runtime stages pageable copies through its own buffers in pieces)
    const size_t in_bytes = (size_t)((unsigned char *)d.x - ctx->d_ws);
    const size_t out_off = in_bytes, out_bytes = (size_t)(p - ctx->d_ws) - in_bytes;
    const bool staged = ensure_stage(ctx, in_bytes + out_bytes);
    pnjl_solve_opts o2 = *opts;
    if (staged) {
        unsigned char *h = ctx->h_stage;
        std::memcpy(h + ((unsigned char *)dT - ctx->d_ws), T, nn * 8);
        std::memcpy(h + ((unsigned char *)du - ctx->d_ws), mu_u, nn * 8);
        std::memcpy(h + ((unsigned char *)dd - ctx->d_ws), mu_d, nn * 8);
        std::memcpy(h + ((unsigned char *)ds - ctx->d_ws), mu_s, nn * 8);
        std::memcpy(h + ((unsigned char *)dxi - ctx->d_ws), xi, nn * 8);
        if (per_point) std::memcpy(h + ((unsigned char *)dseeds - ctx->d_ws), opts->point_seeds, 5 * nn * 8);
        PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_ws, h, in_bytes, cudaMemcpyHostToDevice, s));
    } else {
        PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dT, T, nn * 8, cudaMemcpyHostToDevice, s));
        PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(du, mu_u, nn * 8, cudaMemcpyHostToDevice, s));
        PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dd, mu_d, nn * 8, cudaMemcpyHostToDevice, s));
        PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(ds, mu_s, nn * 8, cudaMemcpyHostToDevice, s));
        PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dxi, xi, nn * 8, cudaMemcpyHostToDevice, s));
        if (per_point)
            PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(dseeds, opts->point_seeds, 5 * nn * 8, cudaMemcpyHostToDevice, s));
    }
    if (per_point) o2.point_seeds = dseeds;
    rc = learned ? pnjl_solve_batch_learned_device(ctx, n, dT, du, dd, ds, dxi, &o2, &d)
                 : pnjl_solve_batch_device(ctx, n, dT, du, dd, ds, dxi, &o2, &d);
    if (rc) return rc;
    if (staged) {
        unsigned char *h = ctx->h_stage;
        PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(h + out_off, ctx->d_ws + out_off, out_bytes, cudaMemcpyDeviceToHost, s));
        PNJL_CUDA_TRY(ctx, cudaStreamSynchronize(s));
        if (out->x) std::memcpy(out->x, h + ((unsigned char *)d.x - ctx->d_ws), (5 * nn) * 8);
        if (out->omega) std::memcpy(out->omega, h + ((unsigned char *)d.omega - ctx->d_ws), (nn) * 8);
        if (out->pressure) std::memcpy(out->pressure, h + ((unsigned char *)d.pressure - ctx->d_ws), (nn) * 8);
        if (out->rho_norm) std::memcpy(out->rho_norm, h + ((unsigned char *)d.rho_norm - ctx->d_ws), (nn) * 8);
        if (out->entropy) std::memcpy(out->entropy, h + ((unsigned char *)d.entropy - ctx->d_ws), (nn) * 8);
        if (out->energy) std::memcpy(out->energy, h + ((unsigned char *)d.energy - ctx->d_ws), (nn) * 8);
        if (out->residual_norm) std::memcpy(out->residual_norm, h + ((unsigned char *)d.residual_norm - ctx->d_ws), (nn) * 8);
        if (out->masses) std::memcpy(out->masses, h + ((unsigned char *)d.masses - ctx->d_ws), (3 * nn) * 8);
        if (out->rho) std::memcpy(out->rho, h + ((unsigned char *)d.rho - ctx->d_ws), (3 * nn) * 8);
        if (out->n_q) std::memcpy(out->n_q, h + ((unsigned char *)d.n_q - ctx->d_ws), (3 * nn) * 8);
        if (out->n_aq) std::memcpy(out->n_aq, h + ((unsigned char *)d.n_aq - ctx->d_ws), (3 * nn) * 8);
        if (out->iterations) std::memcpy(out->iterations, h + ((unsigned char *)d.iterations - ctx->d_ws), (nn) * 4);
        if (out->chosen_seed) std::memcpy(out->chosen_seed, h + ((unsigned char *)d.chosen_seed - ctx->d_ws), (nn) * 4);
        if (out->status) std::memcpy(out->status, h + ((unsigned char *)d.status - ctx->d_ws), (nn) * 4);
        if (out->converged) std::memcpy(out->converged, h + ((unsigned char *)d.converged - ctx->d_ws), (nn) * 1);
    } else {
        if (out->x) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->x, d.x, (5 * nn) * 8, cudaMemcpyDeviceToHost, s));
        if (out->omega) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->omega, d.omega, (nn) * 8, cudaMemcpyDeviceToHost, s));
        if (out->pressure) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->pressure, d.pressure, (nn) * 8, cudaMemcpyDeviceToHost, s));
        if (out->rho_norm) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->rho_norm, d.rho_norm, (nn) * 8, cudaMemcpyDeviceToHost, s));
        if (out->entropy) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->entropy, d.entropy, (nn) * 8, cudaMemcpyDeviceToHost, s));
        if (out->energy) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->energy, d.energy, (nn) * 8, cudaMemcpyDeviceToHost, s));
        if (out->residual_norm) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->residual_norm, d.residual_norm, (nn) * 8, cudaMemcpyDeviceToHost, s));
        if (out->masses) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->masses, d.masses, (3 * nn) * 8, cudaMemcpyDeviceToHost, s));
        if (out->rho) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->rho, d.rho, (3 * nn) * 8, cudaMemcpyDeviceToHost, s));
        if (out->n_q) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->n_q, d.n_q, (3 * nn) * 8, cudaMemcpyDeviceToHost, s));
        if (out->n_aq) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->n_aq, d.n_aq, (3 * nn) * 8, cudaMemcpyDeviceToHost, s));
        if (out->iterations) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->iterations, d.iterations, (nn) * 4, cudaMemcpyDeviceToHost, s));
        if (out->chosen_seed) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->chosen_seed, d.chosen_seed, (nn) * 4, cudaMemcpyDeviceToHost, s));
        if (out->status) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->status, d.status, (nn) * 4, cudaMemcpyDeviceToHost, s));
        if (out->converged) PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(out->converged, d.converged, (nn) * 1, cudaMemcpyDeviceToHost, s));
    }
    PNJL_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    if (pnjl_get_stats(ctx, &ctx->stats) != PNJL_OK) return PNJL_ERR_CUDA;
    if (ctx->stats.device_wait_timeouts)
        return fail(ctx, PNJL_ERR_CUDA, "a solve kernel gave up waiting on a listed point or a plateau bound (results incomplete or not reproducible)");
    return PNJL_OK;
}

int pnjl_solve_batch(pnjl_ctx *ctx, int64_t n, const double *T, const double *mu_u, const double *mu_d,
                     const double *mu_s, const double *xi, const pnjl_solve_opts *opts, pnjl_result_soa *out) {
    return solve_batch_host(ctx, n, T, mu_u, mu_d, mu_s, xi, opts, out, false);
}

int pnjl_solve_batch_learned(pnjl_ctx *ctx, int64_t n, const double *T, const double *mu_u, const double *mu_d,
                             const double *mu_s, const double *xi, const pnjl_solve_opts *opts,
                             pnjl_result_soa *out) {
    return solve_batch_host(ctx, n, T, mu_u, mu_d, mu_s, xi, opts, out, true);
}

void *pnjl_stream(pnjl_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int pnjl_synchronize(pnjl_ctx *ctx) {
    if (!ctx) return PNJL_ERR_INVALID_ARGUMENT;
    PNJL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return PNJL_OK;
}

static void fill_counters(pnjl_stats &st, const long long *c) {
    st.passes_fp64 = c[pnjl::kStatPasses64];
    st.node_evals_fp64_newton = c[pnjl::kStatEvalsNewton64];
    st.node_evals_fp64_thermo = c[pnjl::kStatEvalsThermo64];
    st.node_evals_fp64_grad = c[pnjl::kStatEvalsGrad64];
    st.node_evals_fp64_grad_thermo = c[pnjl::kStatEvalsGradThermo64];
    st.node_evals_fp64 = st.node_evals_fp64_newton + st.node_evals_fp64_thermo + st.node_evals_fp64_grad +
                         st.node_evals_fp64_grad_thermo;
    st.seeds_run = c[pnjl::kStatSeeds];
    st.trust_region_runs = c[pnjl::kStatTrRuns];
    st.multiseed_fallbacks = c[pnjl::kStatMsFallbacks];
    st.passes_fp32 = c[pnjl::kStatPasses32];
    st.node_evals_fp32 = c[pnjl::kStatEvals32];
    st.fp64_rescues = c[pnjl::kStatRescue64];
    st.node_evals_fp32_thermo = c[pnjl::kStatEvalsThermo32];
    st.pruned_candidates = c[pnjl::kStatPruned];
    st.node_evals_ff = c[pnjl::kStatEvalsFF];
    st.node_evals_ff_thermo = c[pnjl::kStatEvalsFFThermo];
    st.device_wait_timeouts = c[pnjl::kStatWaitTimeouts];
    st.node_evals_ff_grad_thermo = c[pnjl::kStatEvalsFFGradThermo];
}

int pnjl_get_stats(const pnjl_ctx *cctx, pnjl_stats *out) {
    pnjl_ctx *ctx = const_cast<pnjl_ctx *>(cctx);
    if (!ctx || !out) return PNJL_ERR_INVALID_ARGUMENT;
    long long h[pnjl::kCtrlSlots];
    PNJL_CUDA_TRY(ctx, cudaMemcpyAsync(h, ctx->d_ctrl, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
    PNJL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    pnjl_stats st = ctx->stats;
    fill_counters(st, h + 1);
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1) == cudaSuccess) st.last_kernel_ms = ms;
    *out = st;
    ctx->stats = st;
    return PNJL_OK;
}

int pnjl_get_kernel_stats(const pnjl_ctx *cctx, int32_t kernel, pnjl_stats *out) {
    pnjl_ctx *ctx = const_cast<pnjl_ctx *>(cctx);
    if (!ctx || !out || (kernel != 0 && kernel != 1)) return PNJL_ERR_INVALID_ARGUMENT;
    pnjl_stats total{};
    int rc = pnjl_get_stats(ctx, &total);
    if (rc) return rc;
    pnjl_stats st = total;
    if (!ctx->split_last) {
        if (kernel == 1) {  // no second kernel: zero work
            pnjl_stats z{};
            z.points = total.points;
            z.kernel_launches = total.kernel_launches;
            *out = z;
            return PNJL_OK;
        }
        *out = total;
        return PNJL_OK;
    }
    long long h[pnjl::kCtrlSlots], t[pnjl::kCtrlSlots];
    PNJL_CUDA_TRY(ctx, cudaMemcpy(h, ctx->d_ctrl_snap, sizeof h, cudaMemcpyDeviceToHost));
    PNJL_CUDA_TRY(ctx, cudaMemcpy(t, ctx->d_ctrl, sizeof t, cudaMemcpyDeviceToHost));
    if (kernel == 1)
        for (int k = 0; k < pnjl::kCtrlSlots; ++k) h[k] = t[k] - h[k];
    fill_counters(st, h + 1);
    float ms = 0.f;
    if (kernel == 0 && cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev_mid) == cudaSuccess) st.last_kernel_ms = ms;
    if (kernel == 1 && cudaEventElapsedTime(&ms, ctx->ev_mid, ctx->ev1) == cudaSuccess) st.last_kernel_ms = ms;
    *out = st;
    return PNJL_OK;
}

int pnjl_device_sm_count(const pnjl_ctx *ctx) { return ctx ? ctx->sm_count : 0; }

extern "C" int pnjl_probe_peak_impl(int device, int kind, double *ops_per_s);
extern "C" int pnjl_f64_math_impl(int device, int fn, int64_t n, const double *x, double *y);

int pnjl_f64_math(pnjl_ctx *ctx, int32_t fn, int64_t n, const double *x, double *y) {
    if (!ctx) return PNJL_ERR_INVALID_ARGUMENT;
    const int rc = pnjl_f64_math_impl(ctx->device, fn, n, x, y);
    if (rc == PNJL_ERR_INVALID_ARGUMENT) return fail(ctx, rc, "pnjl_f64_math: bad arguments");
    return rc;
}

int pnjl_probe_peak(pnjl_ctx *ctx, int32_t kind, double *ops_per_s) {
    if (!ctx) return PNJL_ERR_INVALID_ARGUMENT;
    PNJL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    int rc = pnjl_probe_peak_impl(ctx->device, kind, ops_per_s);
    if (rc) return fail(ctx, rc, "peak probe failed");
    return PNJL_OK;
}

int pnjl_set_pipeline(pnjl_ctx *ctx, int32_t chunks) {
    if (!ctx) return PNJL_ERR_INVALID_ARGUMENT;
    if (chunks < -1 || chunks > pnjl::kMaxPipelineChunks)
        return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "pipeline chunks out of range (-1..16)");
    ctx->pipeline_chunks = chunks;
    return PNJL_OK;
}

int pnjl_set_cert_warps(pnjl_ctx *ctx, int32_t warps) {
    if (!ctx) return PNJL_ERR_INVALID_ARGUMENT;
    if (warps < 0 || warps > pnjl::kFusedThreads / 32 - 1)
        return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "certifying warps out of range (0..7)");
    ctx->cert_warps = warps;
    return PNJL_OK;
}

int pnjl_get_cert_warps(const pnjl_ctx *ctx, int32_t *warps) {
    if (!ctx || !warps) return PNJL_ERR_INVALID_ARGUMENT;
    *warps = ctx->cert_warps;
    return PNJL_OK;
}

int pnjl_set_wait_limits(pnjl_ctx *ctx, uint32_t ready_polls, uint32_t verdict_polls) {
    if (!ctx) return PNJL_ERR_INVALID_ARGUMENT;
    ctx->ready_polls = ready_polls;
    ctx->verdict_polls = verdict_polls;
    return PNJL_OK;
}

int pnjl_get_wait_limits(const pnjl_ctx *ctx, uint32_t *ready_polls, uint32_t *verdict_polls) {
    if (!ctx || !ready_polls || !verdict_polls) return PNJL_ERR_INVALID_ARGUMENT;
    *ready_polls = ctx->ready_polls;
    *verdict_polls = ctx->verdict_polls;
    return PNJL_OK;
}

int pnjl_get_tuning(const pnjl_ctx *ctx, int32_t *lanes_per_point, int32_t *blocks_per_sm, int32_t *chunks) {
    if (!ctx) return PNJL_ERR_INVALID_ARGUMENT;
    if (lanes_per_point) *lanes_per_point = ctx->group;
    if (blocks_per_sm) *blocks_per_sm = ctx->blocks_per_sm;
    if (chunks) *chunks = ctx->pipeline_chunks;
    return PNJL_OK;
}

int pnjl_autotune(pnjl_ctx *ctx, int64_t n, const double *d_T, const double *d_mu_u, const double *d_mu_d,
                  const double *d_mu_s, const double *d_xi, const pnjl_solve_opts *opts, pnjl_result_soa *d_out,
                  int32_t learned, int32_t reps, pnjl_tuning *best, pnjl_tuning *tried, int32_t max_tried,
                  int32_t *n_tried) {
    if (!ctx || !opts || !d_out || !best || n <= 0 || reps < 1) return PNJL_ERR_INVALID_ARGUMENT;
    int rc = check_opts(ctx, opts);
    if (rc) return rc;
    const bool mixed = opts->precision == PNJL_PREC_MIXED;
    const bool per_point = learned || opts->seed_mode == PNJL_SEEDS_PER_POINT;
    int occ_max = mixed ? std::max(pnjl::solve_mixed_occupancy(pnjl::kMixedFused,
                                                               pnjl::node_smem_bytes(ctx->p_num, ctx->t_num)), 1)
                        : std::max(pnjl::solve_kernel_occupancy(32, pnjl::node_smem_bytes(ctx->p_num, ctx->t_num)), 1);
    // launch forms (pipeline chunks, certifying warps): the fused kernel with 0..4 certifying
    // warps per block, the two kernels in sequence, the two-stream chunk pipeline
    const int form_list[][2] = {{1, 0}, {1, 1}, {1, 2}, {1, 3}, {1, 4}, {-1, 0}, {2, 0}, {4, 0}};
    const int n_form = (mixed && per_point) ? 8 : 1;
    const int old_bps = ctx->blocks_per_sm, old_c = ctx->pipeline_chunks, old_k = ctx->cert_warps;
    pnjl_tuning b{};
    b.ms = 1e300;
    int count = 0;
    for (int bps = occ_max; bps >= 1; --bps) {
        for (int ci = 0; ci < n_form; ++ci) {
            ctx->blocks_per_sm = bps;
            ctx->pipeline_chunks = form_list[ci][0];
            ctx->cert_warps = form_list[ci][1];
            double t_min = 1e300;
            for (int r = 0; r < reps; ++r) {
                rc = learned ? pnjl_solve_batch_learned_device(ctx, n, d_T, d_mu_u, d_mu_d, d_mu_s, d_xi, opts, d_out)
                             : pnjl_solve_batch_device(ctx, n, d_T, d_mu_u, d_mu_d, d_mu_s, d_xi, opts, d_out);
                if (rc) {
                    ctx->blocks_per_sm = old_bps;
                    ctx->pipeline_chunks = old_c;
                    ctx->cert_warps = old_k;
                    return rc;
                }
                PNJL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
                float ms = 0.f;
                PNJL_CUDA_TRY(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
                t_min = std::min(t_min, (double)ms);
            }
            pnjl_tuning t{32, bps, form_list[ci][0], form_list[ci][1], t_min};
            if (tried && count < max_tried) tried[count] = t;
            ++count;
            if (t_min < b.ms) b = t;
        }
    }
    if (n_tried) *n_tried = count;
    ctx->blocks_per_sm = b.blocks_per_sm;
    ctx->pipeline_chunks = b.pipeline_chunks;
    ctx->cert_warps = b.pipeline_chunks == 1 || b.pipeline_chunks == 0 ? b.cert_warps : old_k;
    *best = b;
    return PNJL_OK;
}

int pnjl_set_tuning(pnjl_ctx *ctx, int32_t lanes_per_point, int32_t blocks_per_sm) {
    if (!ctx) return PNJL_ERR_INVALID_ARGUMENT;
    if (lanes_per_point != 32)
        return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "lanes_per_point must be 32");
    if (blocks_per_sm < 0 || blocks_per_sm > 32) return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "blocks_per_sm out of range");
    ctx->group = lanes_per_point;
    ctx->blocks_per_sm = blocks_per_sm;
    return PNJL_OK;
}


// ---------------------------------------------------------------------------------------
// Plans: several batched solves -- each with its own quadrature order, inputs, outputs and
// options -- captured once into one CUDA graph and replayed with one launch.

struct PlanSeg {
    int p_num = 0, t_num = 0;
    double *d_nodes = nullptr;
    float *d_nodes_f = nullptr;
    int64_t n = 0;
    const double *T = nullptr, *mu_u = nullptr, *mu_d = nullptr, *mu_s = nullptr, *xi = nullptr;
    pnjl_solve_opts opts{};
    double *d_seeds = nullptr;         // seed tables (cold | hot)
    unsigned char *d_vmap = nullptr;
    double *d_point_seeds = nullptr;   // learned segments: the network's seeds
    bool learned = false;
    pnjl_result_soa out{};
    long long *ctrl = nullptr;
    unsigned char *scratch = nullptr;
    cudaStream_t s = nullptr, s2 = nullptr;
    cudaEvent_t ev_chunk[pnjl::kMaxPipelineChunks] = {};
    cudaEvent_t ev_join = nullptr, ev_done = nullptr;
};

struct pnjl_plan {
    pnjl_ctx *ctx = nullptr;
    std::vector<PlanSeg> segs;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev_fork = nullptr;
    int launches = 0;
};

static void plan_free(pnjl_plan *pl) {
    if (!pl) return;
    if (pl->ctx) cudaSetDevice(pl->ctx->device);
    if (pl->exec) cudaGraphExecDestroy(pl->exec);
    if (pl->graph) cudaGraphDestroy(pl->graph);
    if (pl->ev_fork) cudaEventDestroy(pl->ev_fork);
    for (auto &g : pl->segs) {
        cudaFree(g.d_nodes); cudaFree(g.d_nodes_f); cudaFree(g.d_seeds); cudaFree(g.d_vmap);
        cudaFree(g.d_point_seeds); cudaFree(g.ctrl); cudaFree(g.scratch);
        for (auto &ev : g.ev_chunk) if (ev) cudaEventDestroy(ev);
        if (g.ev_join) cudaEventDestroy(g.ev_join);
        if (g.ev_done) cudaEventDestroy(g.ev_done);
        if (g.s) cudaStreamDestroy(g.s);
        if (g.s2) cudaStreamDestroy(g.s2);
    }
    delete pl;
}

int pnjl_plan_create(pnjl_ctx *ctx, pnjl_plan **out) {
    if (!ctx || !out) return PNJL_ERR_INVALID_ARGUMENT;
    pnjl_plan *pl = new (std::nothrow) pnjl_plan();
    if (!pl) return PNJL_ERR_OUT_OF_MEMORY;
    pl->ctx = ctx;
    *out = pl;
    return PNJL_OK;
}

int pnjl_plan_add(pnjl_plan *pl, int32_t p_num, int32_t t_num, double p_max, int64_t n, const double *d_T,
                  const double *d_mu_u, const double *d_mu_d, const double *d_mu_s, const double *d_xi,
                  const pnjl_solve_opts *opts, int32_t learned, pnjl_result_soa *d_out) {
    if (!pl || !pl->ctx) return PNJL_ERR_INVALID_ARGUMENT;
    pnjl_ctx *ctx = pl->ctx;
    if (pl->exec) return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "plan already finalised");
    int rc = check_opts(ctx, opts);
    if (rc) return rc;
    if (p_num < 1 || p_num > pnjl::kMaxPNodes || t_num < 1 || t_num > pnjl::kMaxTNodes || !(p_max > 0.0))
        return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "node counts out of range (1..512 x 1..64, p_max > 0)");
    if (n <= 0 || !d_out || !d_T || !d_mu_u || !d_mu_d || !d_mu_s || !d_xi)
        return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "segment needs n > 0 points and device arrays");
    if (learned) {
        rc = mlp_require(ctx, true);
        if (rc) return rc;
    }
    cudaSetDevice(ctx->device);
    PlanSeg g;
    g.p_num = p_num;
    g.t_num = t_num;
    g.n = n;
    g.T = d_T; g.mu_u = d_mu_u; g.mu_d = d_mu_d; g.mu_s = d_mu_s; g.xi = d_xi;
    g.opts = *opts;
    g.out = *d_out;
    g.learned = learned != 0;
    std::vector<double> h;
    std::vector<float> hf;
    node_tables_host(p_num, t_num, p_max, h, hf);
    bool ok = cudaMalloc(&g.d_nodes, h.size() * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&g.d_nodes_f, hf.size() * sizeof(float)) == cudaSuccess &&
              cudaMemcpy(g.d_nodes, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(g.d_nodes_f, hf.data(), hf.size() * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess;
    // the seed tables and the verification map are copied now: the graph reads device copies
    ok = ok && cudaMalloc(&g.d_seeds, 2 * 16 * 5 * sizeof(double)) == cudaSuccess &&
         cudaMemset(g.d_seeds, 0, 2 * 16 * 5 * sizeof(double)) == cudaSuccess;
    if (ok && opts->n_seeds > 0 && opts->seed_table) {
        ok = cudaMemcpy(g.d_seeds, opts->seed_table, opts->n_seeds * 5 * sizeof(double), cudaMemcpyHostToDevice) ==
             cudaSuccess;
        if (ok && opts->seed_table_hot)
            ok = cudaMemcpy(g.d_seeds + 80, opts->seed_table_hot, opts->n_seeds * 5 * sizeof(double),
                            cudaMemcpyHostToDevice) == cudaSuccess;
    }
    if (ok && pnjl::verify_map_cells(opts)) {
        const size_t cells = (size_t)pnjl::verify_map_cells(opts);
        ok = cudaMalloc(&g.d_vmap, cells) == cudaSuccess &&
             cudaMemcpy(g.d_vmap, opts->verify_map, cells, cudaMemcpyHostToDevice) == cudaSuccess;
    }
    if (ok && g.learned) {
        ok = cudaMalloc(&g.d_point_seeds, (size_t)n * 5 * sizeof(double)) == cudaSuccess;
        g.opts.seed_mode = PNJL_SEEDS_PER_POINT;
        g.opts.point_seeds = g.d_point_seeds;
    }
    if (ok) {
        const size_t bytes = solve_scratch_bytes(n, &g.opts);
        ok = cudaMalloc(&g.ctrl, pnjl::kCtrlSlots * sizeof(long long)) == cudaSuccess &&
             cudaMemset(g.ctrl, 0, pnjl::kCtrlSlots * sizeof(long long)) == cudaSuccess &&
             (bytes == 0 || cudaMalloc(&g.scratch, bytes) == cudaSuccess);
    }
    ok = ok && cudaStreamCreateWithFlags(&g.s, cudaStreamNonBlocking) == cudaSuccess &&
         cudaStreamCreateWithFlags(&g.s2, cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&g.ev_join, cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreateWithFlags(&g.ev_done, cudaEventDisableTiming) == cudaSuccess;
    for (int k = 0; ok && k < pnjl::kMaxPipelineChunks; ++k)
        ok = cudaEventCreateWithFlags(&g.ev_chunk[k], cudaEventDisableTiming) == cudaSuccess;
    // host pointers of the options are not read after this call
    g.opts.seed_table = opts->n_seeds > 0 && opts->seed_table ? g.d_seeds : nullptr;
    g.opts.seed_table_hot = opts->n_seeds > 0 && opts->seed_table_hot ? g.d_seeds + 80 : nullptr;
    g.opts.verify_map = g.d_vmap;
    if (!ok) {
        pnjl_plan *tmp = new (std::nothrow) pnjl_plan();
        if (tmp) {  // free this segment's resources through the plan destructor
            tmp->ctx = ctx;
            tmp->segs.push_back(g);
            plan_free(tmp);
        }
        return fail(ctx, PNJL_ERR_OUT_OF_MEMORY, "plan segment allocation failed");
    }
    pl->segs.push_back(g);
    return PNJL_OK;
}

int pnjl_plan_finalize(pnjl_plan *pl) {
    if (!pl || !pl->ctx) return PNJL_ERR_INVALID_ARGUMENT;
    pnjl_ctx *ctx = pl->ctx;
    if (pl->exec) return PNJL_OK;
    if (pl->segs.empty()) return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "plan has no segments");
    cudaSetDevice(ctx->device);
    PNJL_CUDA_TRY(ctx, cudaEventCreateWithFlags(&pl->ev_fork, cudaEventDisableTiming));
    PNJL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    // every segment runs on its own stream pair: the graph gets one branch per segment
    cudaStream_t s = ctx->stream;
    PNJL_CUDA_TRY(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaEventRecord(pl->ev_fork, s);
    int launches = 0;
    for (auto &g : pl->segs) {
        if (e == cudaSuccess) e = cudaStreamWaitEvent(g.s, pl->ev_fork, 0);
        if (e == cudaSuccess && g.learned) {
            e = pnjl::mlp_launch_infer(mlp_dev(ctx), ctx->mlp.sc, g.n, g.T, g.mu_u, g.xi, g.d_point_seeds,
                                       ctx->sm_count, g.s);
            ++launches;
        }
        if (e == cudaSuccess) {
            SolveRes r{g.ctrl, g.scratch, g.d_seeds, g.d_vmap, g.s, g.s2, g.ev_chunk, g.ev_join, nullptr, nullptr};
            int l = 0;
            bool split = false;
            e = solve_enqueue(ctx, kernel_nodes_of(g.d_nodes, g.d_nodes_f, g.p_num, g.t_num), g.n, g.T, g.mu_u,
                              g.mu_d, g.mu_s, g.xi, &g.opts, g.out, r, &l, &split);
            launches += l;
        }
        if (e == cudaSuccess) e = cudaEventRecord(g.ev_done, g.s);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, g.ev_done, 0);
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(s, &graph);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return cuda_fail(ctx, e != cudaSuccess ? e : e2, "plan capture");
    }
    pl->graph = graph;
    PNJL_CUDA_TRY(ctx, cudaGraphInstantiate(&pl->exec, graph, 0));
    pl->launches = launches;
    return PNJL_OK;
}

int pnjl_plan_launch(pnjl_plan *pl) {
    if (!pl || !pl->ctx) return PNJL_ERR_INVALID_ARGUMENT;
    pnjl_ctx *ctx = pl->ctx;
    if (!pl->exec) return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "plan not finalised");
    cudaSetDevice(ctx->device);
    PNJL_CUDA_TRY(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    PNJL_CUDA_TRY(ctx, cudaGraphLaunch(pl->exec, ctx->stream));
    PNJL_CUDA_TRY(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    ctx->split_last = false;
    ctx->stats.kernel_launches += pl->launches;
    return PNJL_OK;
}

int pnjl_plan_stats(pnjl_plan *pl, int32_t segment, pnjl_stats *out) {
    if (!pl || !pl->ctx || !out) return PNJL_ERR_INVALID_ARGUMENT;
    pnjl_ctx *ctx = pl->ctx;
    if (segment < -1 || segment >= (int32_t)pl->segs.size()) return fail(ctx, PNJL_ERR_INVALID_ARGUMENT, "no such segment");
    cudaSetDevice(ctx->device);
    PNJL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    pnjl_stats st{};
    long long sum[pnjl::kCtrlSlots] = {};
    for (int k = 0; k < (int)pl->segs.size(); ++k) {
        if (segment >= 0 && k != segment) continue;
        long long h[pnjl::kCtrlSlots];
        PNJL_CUDA_TRY(ctx, cudaMemcpy(h, pl->segs[k].ctrl, sizeof h, cudaMemcpyDeviceToHost));
        for (int j = 0; j < pnjl::kCtrlSlots; ++j) sum[j] += h[j];
        st.points += pl->segs[k].n;
    }
    fill_counters(st, sum + 1);
    st.kernel_launches = pl->launches;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1) == cudaSuccess) st.last_kernel_ms = ms;
    *out = st;
    return PNJL_OK;
}

int pnjl_plan_destroy(pnjl_plan *pl) {
    plan_free(pl);
    return PNJL_OK;
}

}  // extern "C"
