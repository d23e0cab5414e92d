// pnjl_mlp.h -- device structures and launchers of the learned-seed MLP (pnjl_mlp.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace pnjl {
namespace mlp {
constexpr int IN = 3;    // (T, mu, xi)
constexpr int H = 128;   // hidden width
constexpr int OUT = 5;   // (phi_u, phi_d, phi_s, Phi, Phibar)
}  // namespace mlp

constexpr int kParamCount = mlp::H * mlp::IN + mlp::H + 2 * (mlp::H * mlp::H + mlp::H) + mlp::OUT * mlp::H + mlp::OUT;

// Gradient slots of a training step: CTA c of the fwd/bwd kernel sums the gradients of its
// tiles (c, c + slots, ...) into slot c; the slots are then added in slot order.
constexpr int kMaxGradSlots = 256;

// Device view of the network: FP32 masters, gradients and Adam moments (packed
// W1[H][IN], b1, W2[H][H], b2, W3[H][H], b3, W4[OUT][H], b4), BF16 weight copies and the
// per-CTA gradient slots [kMaxGradSlots][kParamCount] and slot losses [kMaxGradSlots].
struct MlpDev {
    float *master, *grad, *adam_m, *adam_v;
    __nv_bfloat16 *w1b, *w2b, *w3b, *w4b;
    float *partial, *loss_part;
};

// Standardisation of inputs (T, mu, xi in fm^-1) and outputs (x in the reference's units).
struct Scaling {
    double in_shift[3], in_scale[3], out_shift[5], out_scale[5];
};

struct TrainBatch {
    const float *x;   // [n][IN] standardised inputs
    const float *y;   // [n][OUT] standardised targets
    const int *perm;  // [epochs][n]: epoch e's permutation of [0, n) at perm + e * n (null: identity)
    long long n;
    int batch;
    long long steps_per_epoch;  // 0: one pass over the first `batch` samples
    long long *step;  // device step counter (incremented at the start of every step)
    float *loss;      // device: loss of the current step
};

struct AdamCfg {
    double lr, lr_min;
    float beta1, beta2, eps;
    long long total_steps;
};

size_t mlp_smem_bytes();
int mlp_grad_slots(int batch);
cudaError_t mlp_setup_attributes();
cudaError_t mlp_launch_step(const MlpDev &m, const TrainBatch &b, const AdamCfg &c, bool update, cudaStream_t s);
cudaError_t mlp_refresh_bf16(const MlpDev &m, cudaStream_t s);
cudaError_t mlp_prepare(const Scaling &sc, long long n, const double *T, const double *mu, const double *xi,
                        const double *targets, float *x, float *y, cudaStream_t s);
cudaError_t mlp_launch_infer(const MlpDev &m, const Scaling &sc, long long n, const double *T, const double *mu,
                             const double *xi, double *seeds, int sm_count, cudaStream_t s);

}  // namespace pnjl
