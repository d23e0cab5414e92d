/*
 * pnjl_cuda.h -- C ABI of libpnjl_cuda, the GB300 (sm_103a) engine for the PNJL
 * gap-equation parameter scan of w5851/Julia_RelaxTime.
 *
 * The reference has no native boundary (it is pure Julia).  These entry points are
 * what its `ccall` shim binds in place of the Julia solver stack; each declaration
 * names the reference function it stands in for.  Conventions:
 *   - plain C types, SoA host (or device) arrays of FP64, int return codes
 *     (PNJL_OK == 0), no exceptions across the boundary;
 *   - units are the reference's: T, mu, M in fm^-1, phi in fm^-3, Omega in fm^-4;
 *   - host buffers are caller-owned; device buffers are owned by the context;
 *   - one context per host thread; every call on a context is serialised on its stream.
 */
#ifndef PNJL_CUDA_H
#define PNJL_CUDA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes ---- */
#define PNJL_OK 0
#define PNJL_ERR_INVALID_ARGUMENT 1
#define PNJL_ERR_CUDA 2
#define PNJL_ERR_NO_NODES 3
#define PNJL_ERR_OUT_OF_MEMORY 4
#define PNJL_ERR_NOT_TRAINED 5
#define PNJL_ERR_TIMEOUT 6
#define PNJL_ERR_TOO_LARGE 7 /* batch beyond the fixed scratch of pnjl_solve_batch_noalloc */

/* ---- per-point status (pnjl_result_soa.status) ---- */
#define PNJL_POINT_CONVERGED 0        /* converged, physical, residual <= residual_norm_max */
#define PNJL_POINT_NOT_CONVERGED 1    /* single-seed result kept, converged == 0            */
#define PNJL_POINT_EXCEPTION 2        /* non-finite residual at the seed (NLsolve raises)   */
#define PNJL_POINT_ALL_SEEDS_FAILED 3 /* solve_multi: "All seeds failed to converge ..."    */
#define PNJL_POINT_INVALID_INPUT 4    /* T <= 0, xi <= -1 or a non-finite input             */

/* ---- seed modes ---- */
#define PNJL_SEEDS_TABLE 0     /* MultiSeed: every row of seed_table, min-Omega selection   */
#define PNJL_SEEDS_PER_POINT 1 /* one seed per point (ContinuitySeed / DefaultSeed / learned),
                                  MultiSeed over seed_table when it fails and
                                  auto_multiseed_fallback != 0                               */

/* ---- arithmetic of the node integrand ---- */
#define PNJL_PREC_FP64 0  /* every pass in FP64 (the plain method)                          */
#define PNJL_PREC_MIXED 1 /* Newton passes with an FP32 Kahan-compensated integrand; the
                             residual that decides convergence, Omega and the thermo output
                             come from FP64 passes                                          */
#define PNJL_PREC_FF_RESIDUAL 2 /* pnjl_eval_batch only: the float-float passes the mixed
                             solver refines with (gradient and Hessian; omega is NaN)       */
#define PNJL_PREC_FP64_CERT 3 /* pnjl_eval_batch only: the FP64 residual pass that certifies
                             the mixed solver's roots (gradient; omega, Hessian NaN)        */
#define PNJL_PREC_FP32_NEWTON 4 /* pnjl_eval_batch only: the FP32 pass of the mixed solver's
                             Newton steps (gradient and Hessian; omega NaN)                 */

/* Model constants in fm units; src/Constants_PNJL.jl:82-103 (hbarc, N_color, rho0,
 * Lambda, G, K, m_ud0, m_s0, T0, a0, a1, a2, b3). */
typedef struct pnjl_params {
    double hbarc_MeV_fm;
    double Lambda;
    double G;
    double K;
    double m_ud0;
    double m_s0;
    double T0;
    double a0, a1, a2, b3;
    double N_color;
    double rho0;
} pnjl_params;

typedef struct pnjl_ctx pnjl_ctx;

/* Options of one batched solve; the fields mirror the keyword arguments of
 * solve(::FixedMu, ...) (src/pnjl/solver/ImplicitSolver.jl:211-223) and the NLsolve
 * tolerances fixed at :112/:144. */
typedef struct pnjl_solve_opts {
    int32_t seed_mode;           /* PNJL_SEEDS_TABLE or PNJL_SEEDS_PER_POINT                  */
    int32_t n_seeds;             /* rows of seed_table (1..16)                               */
    const double *seed_table;    /* [n_seeds*5] host, (phi_u, phi_d, phi_s, Phi, Phibar)     */
    const double *seed_table_hot;/* NULL or [n_seeds*5]: row used instead when T*hbarc >= hot_T_MeV
                                    (DefaultSeed(:quark) -> VERY_HIGH_TEMP, SeedStrategies.jl:212-220) */
    double hot_T_MeV;            /* 300 in the reference                                      */
    const double *point_seeds;   /* [n*5] for PNJL_SEEDS_PER_POINT (same memory space as T)  */
    int32_t max_iter;            /* NLsolve iterations (reference default 1000; scan 40)     */
    double ftol;                 /* 1e-9 in the reference                                     */
    double xtol;                 /* 1e-9                                                      */
    double residual_norm_max;    /* 1e-6                                                      */
    double phi_tol;              /* 1e-8, physicality window of Phi, Phibar                   */
    double omega_tie_rtol;       /* candidates within rtol*|Omega_min| of the minimum count as
                                    tied; the earliest seed wins (0 = strict argmin)           */
    int32_t trust_region_fallback;   /* ImplicitSolver.jl:130-151                            */
    int32_t auto_multiseed_fallback; /* ImplicitSolver.jl:306-327                            */
    int32_t precision;           /* PNJL_PREC_FP64 / PNJL_PREC_MIXED                          */
    int32_t verify_seeds;        /* PNJL_SEEDS_PER_POINT only: a converged per-point solution is
                                    also checked against the first verify_seeds rows of the seed
                                    table at T*hbarc < verify_T_max_MeV (where a first-order line
                                    allows a lower-Omega branch); min-Omega with the per-point
                                    seed first.  Also verified, at any T: a solution on an
                                    unstable branch (det of the Jacobian of grad_x P negative: a
                                    second negative eigenvalue of the Hessian of Omega besides
                                    the Polyakov-loop saddle, so never the min-Omega phase).
                                    0 disables (the reference's single-seed path). */
    double verify_T_max_MeV;
    double verify_max_step;      /* ... and, at any T, when the converged state lies farther than
                                    this (infinity norm) from its per-point seed: the seed did not
                                    predict the branch it converged to.  <= 0 disables. */
    const uint8_t *verify_map;   /* NULL, or host [dims[0]*dims[1]*dims[2]] flags over a uniform
                                    (T, mu_u, xi) cell grid (T, mu in fm^-1, row-major, xi
                                    fastest): when given, it replaces the verify_T_max_MeV rule --
                                    a point is verified when its cell is flagged (points outside
                                    the grid are always verified).  The learned-seed trainer flags
                                    the cells where its labels show two coexisting phases or a
                                    jump of the solution, grown by one cell. */
    int32_t verify_map_dims[3];  /* cells along T, mu, xi (each >= 1)                          */
    double verify_map_lo[3];     /* grid box: lower and upper edges along T, mu, xi            */
    double verify_map_hi[3];
} pnjl_solve_opts;

/* Per-point results, SoA; any NULL pointer skips that output.  Fields follow SolverResult
 * (ImplicitSolver.jl:178-193) plus the number densities of calculate_number_densities
 * (Thermodynamics.jl:255-281) and the per-flavour densities rho_f = dP/dmu_f. */
typedef struct pnjl_result_soa {
    double *x;             /* [5n] solution (phi_u, phi_d, phi_s, Phi, Phibar)       */
    double *omega;         /* [n]                                                    */
    double *pressure;      /* [n]                                                    */
    double *rho_norm;      /* [n]  sum(rho_f)/(3 rho0)                               */
    double *entropy;       /* [n]                                                    */
    double *energy;        /* [n]                                                    */
    double *masses;        /* [3n]                                                   */
    double *rho;           /* [3n]                                                   */
    double *n_q;           /* [3n] quark number densities n_u, n_d, n_s              */
    double *n_aq;          /* [3n] antiquark number densities                        */
    double *residual_norm; /* [n]  ||F||_inf of the chosen candidate                 */
    int32_t *iterations;   /* [n]                                                    */
    int32_t *chosen_seed;  /* [n]  row of seed_table, -1 for the per-point seed      */
    int32_t *status;       /* [n]  PNJL_POINT_*                                      */
    uint8_t *converged;    /* [n]                                                    */
} pnjl_result_soa;

/* Counters of the last solve on the context.  A node-flavour evaluation is one (p, cos(theta),
 * flavour) term of the thermal integral; the kinds differ in what a pass computes. */
typedef struct pnjl_stats {
    int64_t points;
    int64_t passes_fp64;      /* passes over the 3*p*t node-flavour mesh in FP64        */
    int64_t passes_fp32;      /* ... in FP32 (mixed precision)                          */
    int64_t node_evals_fp64;  /* all FP64 node-flavour evaluations                      */
    int64_t node_evals_fp64_newton;      /* residual + Jacobian passes                  */
    int64_t node_evals_fp64_thermo;      /* Omega, entropy, rho, n_f passes             */
    int64_t node_evals_fp64_grad;        /* residual-only passes (mixed refinement)     */
    int64_t node_evals_fp64_grad_thermo; /* residual + thermo passes (mixed refinement) */
    int64_t node_evals_fp32;  /* FP32 residual + Jacobian passes                        */
    int64_t seeds_run;        /* Newton (+ trust region) runs                           */
    int64_t trust_region_runs;
    int64_t multiseed_fallbacks;
    int64_t kernel_launches;
    double last_kernel_ms;    /* device time of the last solve kernel (CUDA events)     */
    int64_t fp64_rescues;     /* mixed mode: FP32-Jacobian refinements that stopped
                                 contracting and were finished by FP64 Newton steps     */
    int64_t node_evals_fp32_thermo; /* mixed mode: FP32 Omega passes at FP32 roots      */
    int64_t pruned_candidates;/* mixed mode: FP32 roots whose Omega lies clearly above a
                                 certified candidate of the same point (they cannot win
                                 the min-Omega selection): no FP64 work spent on them   */
    int64_t node_evals_ff;    /* mixed mode: float-float residual passes (FP32 pipe)    */
    int64_t node_evals_ff_thermo; /* mixed mode: float-float Omega / thermo passes at
                                 certified states (FP32 pipe)                           */
    int64_t device_wait_timeouts; /* mixed mode: tasks that gave up waiting (bounded) on a
                                 listed point still being written; always 0 in practice.
                                 pnjl_solve_batch returns PNJL_ERR_CUDA when it is not. */
    int64_t node_evals_ff_grad_thermo; /* mixed mode: float-float passes giving both the
                                 residual and the outputs (after a correction step)     */
} pnjl_stats;

/* Default parameter set: config/pnjl/default.toml:1-21 through Constants_PNJL.jl:82-103. */
int pnjl_params_default(pnjl_params *out);

/* Context on one GPU; replaces the module-level constants of Constants_PNJL.jl (any
 * profile loaded by load_pnjl_config, :57-73, is passed in here). */
int pnjl_init(const pnjl_params *params, int device, pnjl_ctx **out);
int pnjl_destroy(pnjl_ctx *ctx);
/* Last error message of the context (thread-local to the context). */
const char *pnjl_last_error(const pnjl_ctx *ctx);

/* Gauss-Legendre meshes of cached_nodes(p_num, t_num) (src/pnjl/core/Integrals.jl:87-110,
 * src/integration/GaussLegendre.jl:94-119): p on [0, p_max], cos(theta) on [0, 1] with
 * doubled weights.  1 <= p_num <= 512, 1 <= t_num <= 64. */
int pnjl_set_nodes(pnjl_ctx *ctx, int32_t p_num, int32_t t_num, double p_max);
/* Copy the column-major meshes back (p_num*t_num each; any pointer may be NULL). */
int pnjl_get_nodes(const pnjl_ctx *ctx, double *p_mesh, double *c_mesh, double *coef);

/* Omega, grad_x Omega [5n] and Hessian_x Omega [25n, row-major] at given states:
 * calculate_omega (Thermodynamics.jl:181-195) and the ForwardDiff gradient/Jacobian of
 * gap_conditions (Conditions.jl:72-86; F = -grad_x Omega).  precision: PNJL_PREC_FP64,
 * PNJL_PREC_MIXED (FP32-Kahan integrand, FP64 assembly), PNJL_PREC_FF_RESIDUAL (float-float
 * gradient and Hessian), PNJL_PREC_FP64_CERT (gradient from the certification pass) or
 * PNJL_PREC_FP32_NEWTON (the mixed solver's FP32 Newton pass).  Host pointers; NULL skips. */
int pnjl_eval_batch(pnjl_ctx *ctx, int64_t n, const double *x, const double *T,
                    const double *mu_u, const double *mu_d, const double *mu_s,
                    const double *xi, int32_t precision,
                    double *omega, double *grad, double *hess);

/* calculate_thermo + calculate_number_densities at given states
 * (Thermodynamics.jl:233-244, :255-281).  Host pointers; fills pressure, rho_norm,
 * entropy, energy, masses, rho, n_q, n_aq and omega of `out` (other fields untouched). */
int pnjl_thermo_batch(pnjl_ctx *ctx, int64_t n, const double *x, const double *T,
                      const double *mu_u, const double *mu_d, const double *mu_s,
                      const double *xi, pnjl_result_soa *out);

/* Batched solve(::FixedMu, T, mu; xi, seed_strategy, ...) over n points
 * (ImplicitSolver.jl:211-328, solve_multi :532-559), flavour-resolved chemical
 * potentials (Conditions.jl:205 takes mu_vec).  Host pointers, synchronous: the timed
 * region of a caller includes the host<->device copies. */
int pnjl_solve_batch(pnjl_ctx *ctx, int64_t n, const double *T, const double *mu_u,
                     const double *mu_d, const double *mu_s, const double *xi,
                     const pnjl_solve_opts *opts, pnjl_result_soa *out);

/* Same with device pointers (inputs and outputs already in HBM); asynchronous on the
 * context stream (see pnjl_stream).  opts->seed_table stays a host pointer;
 * opts->point_seeds is a device pointer here. */
int pnjl_solve_batch_device(pnjl_ctx *ctx, int64_t n, const double *d_T, const double *d_mu_u,
                            const double *d_mu_d, const double *d_mu_s, const double *d_xi,
                            const pnjl_solve_opts *opts, pnjl_result_soa *d_out);

/* The context's CUDA stream (a cudaStream_t) and a blocking wait on it. */
void *pnjl_stream(pnjl_ctx *ctx);
int pnjl_synchronize(pnjl_ctx *ctx);
int pnjl_get_stats(const pnjl_ctx *ctx, pnjl_stats *out);
/* The same for one kernel of the last solve: kernel 0 = the first kernel (the per-point kernel
 * of a mixed per-point solve run as two kernels, else the only one), kernel 1 = the task
 * kernel that follows it (all counters zero when there was none).  last_kernel_ms is that
 * kernel's device time (CUDA events around it on the context stream). */
int pnjl_get_kernel_stats(const pnjl_ctx *ctx, int32_t kernel, pnjl_stats *out);

/* Number of streaming multiprocessors of the context's device. */
int pnjl_device_sm_count(const pnjl_ctx *ctx);

/* Launch shape of the solve kernel: lanes per task (32: one warp) and resident blocks
 * per SM (0 = occupancy maximum).  Chosen by the autotuner; results do not depend on it. */
int pnjl_set_tuning(pnjl_ctx *ctx, int32_t lanes_per_point, int32_t blocks_per_sm);
/* How a mixed-precision per-point solve (learned / continuation seeds) with a MultiSeed table
 * is launched.  1 (and 0, automatic): one fused kernel, in which the verification and
 * MultiSeed-fallback tasks of listed points run beside the remaining points.  -1: the per-point
 * kernel, then the task kernel (pnjl_get_kernel_stats splits their counters and times).
 * 2..16: the points are cut into that many pieces over two streams, and the task kernel of
 * piece c overlaps the per-point kernel of piece c+1.  Results do not depend on it.
 * pnjl_get_tuning reads the current launch shape. */
int pnjl_set_pipeline(pnjl_ctx *ctx, int32_t chunks);
/* Certifying warps per block of the fused kernel (0..7; 0 by default): these warps run only
 * the FP64 certification passes that the other warps queue, a steady supply of work for the
 * FP64 pipe.  0: every warp certifies its own seeds (measured fastest on the 256 x 256 x 9
 * scan; the autotuner tries 0..4).  Results do not depend on it. */
int pnjl_set_cert_warps(pnjl_ctx *ctx, int32_t warps);
int pnjl_get_cert_warps(const pnjl_ctx *ctx, int32_t *warps);
/* Bounds of the fused kernel's waits (no counterpart in the reference, which has no GPU code):
 * a warp that has taken a listed slot's task or a queued certification polls the entry's
 * ready flag, written by a running warp of the same launch, at most ready_polls times (64 ns
 * apart; default 2^24, about 1 s); a seed whose FP32 root an earlier seed is still certifying
 * polls that verdict at most verdict_polls times (128 ns apart; default 2^20), and so does a
 * seed of a point without a per-point root that reaches a residual plateau and waits for seed
 * 0's verdict (its plateau bound).  A ready wait that runs out leaves the task undone, a
 * seed-0 wait that runs out leaves the seed without a bound; both are counted in
 * pnjl_stats.device_wait_timeouts, and the host-array solves then return PNJL_ERR_CUDA
 * (results incomplete, or not reproducible) -- the context stays usable; a verdict wait that runs out makes the
 * waiting seed certify the root itself (same result).  0 means no polls: a flag not set at
 * the first read gives up at once. */
int pnjl_set_wait_limits(pnjl_ctx *ctx, uint32_t ready_polls, uint32_t verdict_polls);
int pnjl_get_wait_limits(const pnjl_ctx *ctx, uint32_t *ready_polls, uint32_t *verdict_polls);
int pnjl_get_tuning(const pnjl_ctx *ctx, int32_t *lanes_per_point, int32_t *blocks_per_sm, int32_t *chunks);

/* One launch shape and its measured solve time (device time of the solve kernels, CUDA events). */
typedef struct pnjl_tuning {
    int32_t lanes_per_point;
    int32_t blocks_per_sm;
    int32_t pipeline_chunks;
    int32_t cert_warps;     /* certifying warps per block of the fused kernel */
    double ms;
} pnjl_tuning;

/* Autotuner (no counterpart in the reference): solves the given representative batch (device
 * pointers, as pnjl_solve_batch_device, or pnjl_solve_batch_learned_device when `learned`) with
 * every candidate launch shape -- resident blocks per SM from the occupancy maximum down to 1,
 * and for mixed per-point solves the fused kernel with 0..4 certifying warps and the launch
 * forms -1, 2, 4 of pnjl_set_pipeline -- `reps` times each, keeps
 * the fastest (minimum over repetitions) and sets it on the context.  `tried` (optional) receives
 * up to max_tried candidates with their times; d_out receives the last solve's results. */
int pnjl_autotune(pnjl_ctx *ctx, int64_t n, const double *d_T, const double *d_mu_u, const double *d_mu_d,
                  const double *d_mu_s, const double *d_xi, const pnjl_solve_opts *opts, pnjl_result_soa *d_out,
                  int32_t learned, int32_t reps, pnjl_tuning *best, pnjl_tuning *tried, int32_t max_tried,
                  int32_t *n_tried);

/* Measured pipe throughput of the context's device, the denominators of the kernels'
 * rooflines (no counterpart in the reference, which has no GPU): kind 0 = FP64 FMA
 * (FLOP/s, FMA = 2), 1 = FP32 FMA (FLOP/s), 2 = SFU ex2.approx.f32 (operations/s), 3 = FP64 FMA
 * issued by one lane per warp (FLOP/s of the active lanes). */
int pnjl_probe_peak(pnjl_ctx *ctx, int32_t kind, double *ops_per_s);

/* Element-wise functions of the mixed solver's passes, for checking them against the library
 * functions (no counterpart in the reference): y[i] = f(x[i]) on the device, host arrays of
 * n.  fn 0: e^x by the FP64 table method (for -700 <= x <= 0; other x take the library exp),
 * 1: 1/x from the hardware approximation and a Newton correction, 2: 1/sqrt(x) likewise; 3,
 * 4, 5: the library exp, division and rsqrt; 6, 7: the float-float e^x and ln x of x rounded
 * to a float pair (hi + lo returned). */
int pnjl_f64_math(pnjl_ctx *ctx, int32_t fn, int64_t n, const double *x, double *y);

/* ---- learned seed: MLP (T, mu, xi) -> (phi_u, phi_d, phi_s, Phi, Phibar) ----------------
 * 3 -> 128 -> 128 -> 128 -> 5, SiLU, BF16 weights, FP32 accumulation, trained with Adam by
 * the library's own BF16 tensor-core kernels on solutions the solver produced.  It replaces
 * the initial guess of get_seed(::SeedStrategy, ...) (src/pnjl/solver/SeedStrategies.jl:118):
 * the reference has no learned seed, so these entry points have no single reference
 * counterpart; the multi-seed solve stays their fallback (pnjl_solve_batch_learned*). */

/* Number of FP32 parameters (packed W1[128][3], b1, W2[128][128], b2, W3, b3, W4[5][128], b4). */
int pnjl_mlp_param_count(void);
/* (Re)initialise the weights (Kaiming-uniform from `seed`) and clear the optimiser state. */
int pnjl_mlp_init(pnjl_ctx *ctx, uint64_t seed);
/* Standardisation: input k = (v_k - in_shift[k]) / in_scale[k] for (T, mu, xi) in fm^-1,
 * output x_j = y_j * out_scale[j] + out_shift[j]. */
int pnjl_mlp_set_scaling(pnjl_ctx *ctx, const double *in_shift, const double *in_scale, const double *out_shift,
                         const double *out_scale);
/* Train on n labelled points (host arrays; targets [n*5]); Adam with a cosine-decayed learning
 * rate over epochs x ceil(n/batch) steps, one CUDA graph replay per step; batch is a multiple
 * of 32; last_loss receives the mean squared standardised error of the final step. */
int pnjl_mlp_train(pnjl_ctx *ctx, int64_t n, const double *T, const double *mu, const double *xi,
                   const double *targets, int32_t epochs, int32_t batch, double lr, uint64_t shuffle_seed,
                   double *last_loss);
/* Loss and gradient (FP32, packed like the parameters) over n points without an update. */
int pnjl_mlp_loss_grad(pnjl_ctx *ctx, int64_t n, const double *T, const double *mu, const double *xi,
                       const double *targets, double *loss, float *grad);
/* Seeds [n*5] for n points: host arrays (synchronous) or device arrays (asynchronous). */
int pnjl_mlp_infer(pnjl_ctx *ctx, int64_t n, const double *T, const double *mu, const double *xi, double *seeds);
int pnjl_mlp_infer_device(pnjl_ctx *ctx, int64_t n, const double *d_T, const double *d_mu, const double *d_xi,
                          double *d_seeds);
/* Read or replace the FP32 parameters (count = pnjl_mlp_param_count()). */
int pnjl_mlp_get_params(pnjl_ctx *ctx, float *out, int64_t count);
int pnjl_mlp_set_params(pnjl_ctx *ctx, const float *in, int64_t count);
/* Learned-seed solve on device arrays: the network's seed per point, then
 * pnjl_solve_batch_device in PNJL_SEEDS_PER_POINT mode with opts' MultiSeed table as the
 * fallback when the learned seed does not give a converged physical solution
 * (solve(FixedMu) with auto_multiseed_fallback, ImplicitSolver.jl:306-327). */
int pnjl_solve_batch_learned_device(pnjl_ctx *ctx, int64_t n, const double *d_T, const double *d_mu_u,
                                    const double *d_mu_d, const double *d_mu_s, const double *d_xi,
                                    const pnjl_solve_opts *opts, pnjl_result_soa *d_out);
/* Same with host pointers, synchronous (the end-to-end call: the host<->device copies of
 * the inputs and results are part of it, like pnjl_solve_batch). */
int pnjl_solve_batch_learned(pnjl_ctx *ctx, int64_t n, const double *T, const double *mu_u,
                             const double *mu_d, const double *mu_s, const double *xi,
                             const pnjl_solve_opts *opts, pnjl_result_soa *out);

/* ---- plans: several batched solves in one CUDA graph ---------------------------------------
 * A plan holds segments -- batched solves, each with its own quadrature order (p_num x t_num
 * on [0, p_max]), device inputs and outputs, options and seed mode (learned: the network's
 * seed per point, as pnjl_solve_batch_learned_device) -- captured once into one CUDA graph
 * with one branch per segment, then replayed by pnjl_plan_launch on the context stream.  No
 * counterpart in the reference (one point at a time, one quadrature per call).  pnjl_plan_add
 * copies the node tables, seed tables and verification map and allocates the segment's
 * scratch, so launches allocate and copy nothing.  Segments write only their own outputs;
 * replays re-read the inputs and (for learned segments) the network weights at launch time.
 * pnjl_plan_stats sums the counters of one segment (or all: segment = -1); last_kernel_ms is
 * the last launch's device time. */
typedef struct pnjl_plan pnjl_plan;
int pnjl_plan_create(pnjl_ctx *ctx, pnjl_plan **out);
int pnjl_plan_add(pnjl_plan *plan, int32_t p_num, int32_t t_num, double p_max, int64_t n, const double *d_T,
                  const double *d_mu_u, const double *d_mu_d, const double *d_mu_s, const double *d_xi,
                  const pnjl_solve_opts *opts, int32_t learned, pnjl_result_soa *d_out);
int pnjl_plan_finalize(pnjl_plan *plan);
int pnjl_plan_launch(pnjl_plan *plan);
int pnjl_plan_stats(pnjl_plan *plan, int32_t segment, pnjl_stats *out);
int pnjl_plan_destroy(pnjl_plan *plan);

/* ---- K data of the relaxation-time chain ----------------------------------------------------
 * build_K_data (scripts/relaxtime/run_gap_transport_scan.jl:297-305) for n solved points: the
 * one-loop integral A_f = OneLoopIntegrals.A(m_f, mu_f, T, Phi, Phibar, nodes, weights)
 * (src/relaxtime/OneLoopIntegrals.jl:507-543) on the p_num Gauss-Legendre nodes of [0, p_max]
 * (the script uses DEFAULT_MOMENTUM_NODES: 64 on [0, 10]), G^f = calculate_G_from_A(A_f, m_f)
 * (src/relaxtime/EffectiveCouplings.jl:56-60) and calculate_effective_couplings(G, K, G^u, G^s)
 * (:242-279) with its determinants (:112-115).  Inputs per point: T, mu_u (used for u and d),
 * mu_s (the script passes one quark chemical potential: pass mu_u again), masses [3n] and
 * the solution x [5n] (Phi = x[3], Phibar = x[4]) -- the layout of pnjl_result_soa.  Any
 * NULL output pointer skips that field.  FP64. */
typedef struct pnjl_kdata_soa {
    double *A_u, *A_d, *A_s;          /* [n] one-loop A per flavour (A_d = A_u, as build_K_data) */
    double *G_u, *G_s;                /* [n] G^f = -N_c/(4 pi^2) m_f A_f                         */
    double *K0_plus, *K0_minus;       /* [n] effective couplings K_alpha^+- (fm^2)               */
    double *K123_plus, *K123_minus;
    double *K4567_plus, *K4567_minus;
    double *K8_plus, *K8_minus;
    double *K08_plus, *K08_minus;
    double *det_K_plus, *det_K_minus; /* [n] K0 K8 - K08^2 per channel (fm^4)                    */
} pnjl_kdata_soa;
/* Host arrays, synchronous. */
int pnjl_kdata_batch(pnjl_ctx *ctx, int64_t n, int32_t p_num, double p_max, const double *T,
                     const double *mu_u, const double *mu_s, const double *masses, const double *x,
                     pnjl_kdata_soa *out);
/* Device arrays, asynchronous on pnjl_stream(ctx) (e.g. straight from a solve's outputs). */
int pnjl_kdata_batch_device(pnjl_ctx *ctx, int64_t n, int32_t p_num, double p_max, const double *d_T,
                            const double *d_mu_u, const double *d_mu_s, const double *d_masses,
                            const double *d_x, pnjl_kdata_soa *d_out);

/* ---- implicit derivatives of solved states ---------------------------------------------------
 * src/pnjl/derivatives/ThermoDerivatives.jl: mass_derivatives (order 1, :132-173),
 * thermo_derivatives (:184-249) and bulk_viscosity_coefficients (:342-465) at n solved states
 * x [5n] (the solution of a pnjl_solve_batch* call at the same T, mu, xi and the context's
 * nodes).  theta = (T, mu) with every mu_f moved together (the reference's mu_u = mu_d = mu_s
 * = mu); dx/dtheta = -(Hessian_x Omega)^-1 d(grad_x Omega)/dtheta (the implicit function
 * theorem the reference applies with ImplicitDifferentiation.jl), then the chain rule.
 * Analytic second derivatives, FP64.  Any NULL output pointer skips that field.  With unequal
 * mu_f, eps's mu term uses their mean (the reference never calls these with unequal mu_f). */
typedef struct pnjl_deriv_soa {
    double *dx_dT, *dx_dmu;           /* [5n] dx/dT, dx/dmu                                    */
    double *dM_dT, *dM_dmu;           /* [3n] dM_f/dT, dM_f/dmu_q (dM/dmu_B = dM/dmu_q / 3)    */
    double *s, *n_B;                  /* [n]  entropy -dOmega/dT, baryon density sum(rho_f)/3  */
    double *ds_dT, *ds_dmu, *dn_dT, *dn_dmu;          /* [n] total derivatives through x(theta) */
    double *pressure, *dP_dT, *dP_dmu;                /* [n]                                    */
    double *energy, *deps_dT, *deps_dmu;              /* [n] eps = -P + sum mu_f rho_f + T s    */
    double *dP_deps_n, *dP_dn_eps;    /* [n] thermo_derivatives' dP/deps|n and dP/dn|eps      */
    double *v_n_sq, *dmuB_dT_sigma;   /* [n] bulk_viscosity_coefficients' v_n^2, dmu_B/dT|s/n  */
} pnjl_deriv_soa;
/* Host arrays, synchronous. */
int pnjl_derivs_batch(pnjl_ctx *ctx, int64_t n, const double *x, const double *T, const double *mu_u,
                      const double *mu_d, const double *mu_s, const double *xi, pnjl_deriv_soa *out);
/* Device arrays, asynchronous on pnjl_stream(ctx). */
int pnjl_derivs_batch_device(pnjl_ctx *ctx, int64_t n, const double *d_x, const double *d_T,
                             const double *d_mu_u, const double *d_mu_d, const double *d_mu_s,
                             const double *d_xi, pnjl_deriv_soa *d_out);

/* Largest batch of pnjl_solve_batch_noalloc, counted in tasks: n * n_seeds in
 * PNJL_SEEDS_TABLE mode, n in PNJL_SEEDS_PER_POINT mode (and n itself at most this). */
#define PNJL_NOALLOC_MAX_TASKS 32768

/* Batched solve that allocates nothing (no counterpart in the reference, which has no GPU
 * code; it is an allocation-free twin of pnjl_solve_batch_device for the plain FP64 solve).
 * For callers that may not allocate device memory when they solve: hosts whose device memory
 * belongs to another allocator's pool that must account for every byte, and services that
 * reserve all memory at start-up so that no later call can fail for lack of it.  They pass
 * device inputs and outputs (same layout and meaning as pnjl_solve_batch_device;
 * opts->seed_table stays a host pointer, opts->point_seeds is a device pointer) and a stream;
 * no context is used and the call makes no cudaMalloc, cudaFree or other allocating call.
 * Two options of pnjl_solve_batch_device are not available and return
 * PNJL_ERR_INVALID_ARGUMENT: opts->verify_map must be NULL, and opts->precision must be
 * PNJL_PREC_FP64 (the mixed-precision solver needs scratch this fixed array does not hold).  The scratch it needs (candidate records, completion
 * counters, queue head, node and seed tables) is one static device array of about 6 MB that
 * every GPU loading this library holds until exit; batches beyond PNJL_NOALLOC_MAX_TASKS
 * tasks return PNJL_ERR_TOO_LARGE.  The call is asynchronous on `stream` (NULL = the legacy
 * default stream) and runs on the current device.  Its first call on a device also looks up
 * the array's device address (cudaGetSymbolAddress) and loads the kernel module.  All calls
 * share the one array and it keeps the last
 * call's contents (the counters are cleared by each call): calls that overlap on the GPU --
 * on two streams, or from two threads -- race and must not be issued. */
int pnjl_solve_batch_noalloc(const pnjl_params *params, int32_t p_num, int32_t t_num, double p_max, int64_t n,
                             const double *d_T, const double *d_mu_u, const double *d_mu_d, const double *d_mu_s,
                             const double *d_xi, const pnjl_solve_opts *opts, pnjl_result_soa *d_out,
                             void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PNJL_CUDA_H */
