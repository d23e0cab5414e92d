// pnjl_mlp.cu -- the learned seed: an MLP (T, mu, xi) -> (phi_u, phi_d, phi_s, Phi, Phibar),
// 3 -> 128 -> 128 -> 128 -> 5 with SiLU, BF16 weights and FP32 accumulation, trained and run
// on the GPU by the kernels in this file.  It stands in for the MultiSeed /
// PhaseAwareContinuitySeed initial guess (src/pnjl/solver/SeedStrategies.jl) and is
// trained on solutions the GPU solver itself produces.
//
//   mlp_fwd_bwd_kernel   32-sample tiles: forward, loss, backward; the two 128x128 layers
//                        (forward, input gradient and weight gradient) run on the tensor
//                        cores as mma.sync m16n8k16 BF16 x BF16 -> FP32 tiles with operands
//                        staged in shared memory; the 3- and 5-wide layers are FP32 SIMT
//                        loops over the same BF16-rounded weights.  CTA c takes tiles
//                        c, c + grid, ... and keeps the sum of their gradients (and losses)
//                        in its own slot of a partial-gradient buffer: no atomics.
//   mlp_update_kernel    per parameter: the slots summed in slot order (a fixed order, so a
//                        training run is bit-reproducible), Adam on the FP32 master, the
//                        BF16 copy refreshed; the step's loss from the slot losses.
//   mlp_reduce_kernel    the slot sums alone (gradient and loss of one batch, no update).
//   mlp_infer_kernel     forward only; writes de-standardised seeds for the solver.
// One epoch of training steps (step counter, fwd/bwd, update) is captured once in a CUDA
// graph and replayed once per epoch; the epochs' sample permutations are uploaded up front.
#include <cmath>
#include <cstring>
#include <cuda_bf16.h>

#include "pnjl_mlp.h"

namespace pnjl {
namespace mlp {

constexpr int TILE = 32;        // samples per CTA
constexpr int NT = 128;         // threads per CTA (4 warps)
constexpr int LDH = H + 8;      // padded BF16 row stride in shared memory (272 bytes)

// parameter packing (FP32 masters, gradients, Adam moments)
constexpr int OFF_W1 = 0;                  // [H][IN]
constexpr int OFF_B1 = OFF_W1 + H * IN;    // [H]
constexpr int OFF_W2 = OFF_B1 + H;         // [H][H]   (out, in)
constexpr int OFF_B2 = OFF_W2 + H * H;
constexpr int OFF_W3 = OFF_B2 + H;
constexpr int OFF_B3 = OFF_W3 + H * H;
constexpr int OFF_W4 = OFF_B3 + H;         // [OUT][H]
constexpr int OFF_B4 = OFF_W4 + OUT * H;
static_assert(OFF_B4 + OUT == kParamCount, "parameter packing");

struct SmemLayout {
    static constexpr size_t W2 = 0;                                   // bf16 [H][LDH]
    static constexpr size_t W3 = W2 + (size_t)H * LDH * 2;            // bf16 [H][LDH]
    static constexpr size_t Z1 = W3 + (size_t)H * LDH * 2;            // f32 [TILE][H]
    static constexpr size_t Z2 = Z1 + (size_t)TILE * H * 4;
    static constexpr size_t Z3 = Z2 + (size_t)TILE * H * 4;
    static constexpr size_t H1 = Z3 + (size_t)TILE * H * 4;           // bf16 [TILE][LDH]
    static constexpr size_t H2 = H1 + (size_t)TILE * LDH * 2;
    static constexpr size_t H3 = H2 + (size_t)TILE * LDH * 2;
    static constexpr size_t W1 = H3 + (size_t)TILE * LDH * 2;         // f32 [H][IN]
    static constexpr size_t W4 = W1 + (size_t)H * IN * 4;             // f32 [OUT][H]
    static constexpr size_t BIAS = W4 + (size_t)OUT * H * 4;          // f32 b1,b2,b3 [H], b4 [OUT]
    static constexpr size_t X = BIAS + (size_t)(3 * H + OUT + 3) * 4; // f32 [TILE][IN]
    static constexpr size_t Y = X + (size_t)TILE * IN * 4;            // f32 [TILE][OUT]
    static constexpr size_t DO = Y + (size_t)TILE * OUT * 4;          // f32 [TILE][OUT]
    static constexpr size_t RED = DO + (size_t)TILE * OUT * 4;        // f32 [NT] reduction scratch
    static constexpr size_t TOTAL = RED + (size_t)NT * 4;
};

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
    const float s = 1.0f / (1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}
__device__ __forceinline__ float bf16r(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// mma.m16n8k16 operand fragments from shared memory with arbitrary element strides:
// A(m, k) = a[m*ras + k*cas] (16x16 tile at m0, k0), B(k, n) = b[k*rbs + n*cbs] (16x8 at k0, n0).
// Register contents follow the PTX ISA fragment layout of mma.m16n8k16 with .bf16 operands.
__device__ __forceinline__ void load_a(const __nv_bfloat16 *a, int ras, int cas, int m0, int k0, uint32_t (&r)[4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int r0 = m0 + g, r1 = m0 + g + 8, c0 = k0 + 2 * t, c1 = k0 + 2 * t + 8;
    r[0] = pack2(a[r0 * ras + c0 * cas], a[r0 * ras + (c0 + 1) * cas]);
    r[1] = pack2(a[r1 * ras + c0 * cas], a[r1 * ras + (c0 + 1) * cas]);
    r[2] = pack2(a[r0 * ras + c1 * cas], a[r0 * ras + (c1 + 1) * cas]);
    r[3] = pack2(a[r1 * ras + c1 * cas], a[r1 * ras + (c1 + 1) * cas]);
}
__device__ __forceinline__ void load_b(const __nv_bfloat16 *b, int rbs, int cbs, int k0, int n0, uint32_t (&r)[2]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int n = n0 + g, k = k0 + 2 * t;
    r[0] = pack2(b[k * rbs + n * cbs], b[(k + 1) * rbs + n * cbs]);
    r[1] = pack2(b[(k + 8) * rbs + n * cbs], b[(k + 9) * rbs + n * cbs]);
}
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// C[TILE x H] = A[TILE x H] . B[H x H] on the tensor cores: warp w owns rows 16*(w&1) .. +15
// and columns 64*(w>>1) .. +63 (8 n-tiles).  acc receives the FP32 tile fragments.
__device__ __forceinline__ void gemm_tile_x_h(const __nv_bfloat16 *A, int ras, int cas, const __nv_bfloat16 *B,
                                              int rbs, int cbs, float (&acc)[8][4]) {
    const int w = threadIdx.x >> 5;
    const int m0 = 16 * (w & 1), nb = 64 * (w >> 1);
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll
    for (int k0 = 0; k0 < H; k0 += 16) {
        uint32_t ra[4];
        load_a(A, ras, cas, m0, k0, ra);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            uint32_t rb[2];
            load_b(B, rbs, cbs, k0, nb + 8 * j, rb);
            mma_bf16(acc[j], ra, rb);
        }
    }
}

// element (row, col) of fragment j of the warp's tile (see gemm_tile_x_h)
__device__ __forceinline__ void frag_coord(int j, int e, int &row, int &col) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    row = 16 * (w & 1) + g + (e >= 2 ? 8 : 0);
    col = 64 * (w >> 1) + 8 * j + 2 * t + (e & 1);
}

// Accumulate one tile's gradient entry into the CTA's slot: the slot's first tile stores,
// later tiles add (each entry has exactly one writer in the CTA, so no atomics are needed).
__device__ __forceinline__ void slot_acc(float *p, float v, bool first) { *p = first ? v : *p + v; }

// Weight gradient G[H x H] of the tile (K = TILE samples): G = D^T . Hin with D(m=out,
// k=sample) = d[k*LDH + m], Hin(k=sample, n=in) = h[k*LDH + n].  Warp w owns output rows
// 32w..32w+31 in two passes of 64 columns; results go to the CTA's gradient slot.
__device__ __forceinline__ void weight_grad(const __nv_bfloat16 *d, const __nv_bfloat16 *h, float *gW, bool first) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll 1
    for (int half = 0; half < 2; ++half) {
        float acc[2][8][4];
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[i][j][0] = acc[i][j][1] = acc[i][j][2] = acc[i][j][3] = 0.f;
#pragma unroll
        for (int k0 = 0; k0 < TILE; k0 += 16) {
            uint32_t ra[2][4];
#pragma unroll
            for (int i = 0; i < 2; ++i) load_a(d, 1, LDH, 32 * w + 16 * i, k0, ra[i]);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                uint32_t rb[2];
                load_b(h, LDH, 1, k0, 64 * half + 8 * j, rb);
#pragma unroll
                for (int i = 0; i < 2; ++i) mma_bf16(acc[i][j], ra[i], rb);
            }
        }
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j)
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int row = 32 * w + 16 * i + g + (e >= 2 ? 8 : 0);
                    const int col = 64 * half + 8 * j + 2 * t + (e & 1);
                    slot_acc(&gW[row * H + col], acc[i][j][e], first);
                }
    }
}

// Block sum of v (fixed tree order) accumulated into *dst by thread 0.
__device__ __forceinline__ void block_reduce_acc(float v, float *red, float *dst, bool first) {
    red[threadIdx.x] = v;
    __syncthreads();
    for (int s = NT / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) slot_acc(dst, red[0], first);
    __syncthreads();
}

// Load the weights and one tile of inputs; forward pass into z*/h* and `out`.
__device__ void forward_tile(const MlpDev &m, const float *xin, int valid, unsigned char *smem, float *out) {
    __nv_bfloat16 *W2s = (__nv_bfloat16 *)(smem + SmemLayout::W2);
    __nv_bfloat16 *W3s = (__nv_bfloat16 *)(smem + SmemLayout::W3);
    float *Z1 = (float *)(smem + SmemLayout::Z1), *Z2 = (float *)(smem + SmemLayout::Z2),
          *Z3 = (float *)(smem + SmemLayout::Z3);
    __nv_bfloat16 *H1 = (__nv_bfloat16 *)(smem + SmemLayout::H1), *H2 = (__nv_bfloat16 *)(smem + SmemLayout::H2),
                  *H3 = (__nv_bfloat16 *)(smem + SmemLayout::H3);
    float *W1s = (float *)(smem + SmemLayout::W1), *W4s = (float *)(smem + SmemLayout::W4);
    float *bias = (float *)(smem + SmemLayout::BIAS);
    const float *X = (const float *)xin;
    for (int i = threadIdx.x; i < H * H; i += NT) {
        const int r = i / H, c = i % H;
        W2s[r * LDH + c] = m.w2b[i];
        W3s[r * LDH + c] = m.w3b[i];
    }
    for (int i = threadIdx.x; i < H * IN; i += NT) W1s[i] = __bfloat162float(m.w1b[i]);
    for (int i = threadIdx.x; i < OUT * H; i += NT) W4s[i] = __bfloat162float(m.w4b[i]);
    for (int i = threadIdx.x; i < H; i += NT) {
        bias[i] = m.master[OFF_B1 + i];
        bias[H + i] = m.master[OFF_B2 + i];
        bias[2 * H + i] = m.master[OFF_B3 + i];
    }
    if (threadIdx.x < OUT) bias[3 * H + threadIdx.x] = m.master[OFF_B4 + threadIdx.x];
    __syncthreads();
    // layer 1 (3 -> 128), FP32 SIMT
    for (int i = threadIdx.x; i < TILE * H; i += NT) {
        const int s = i / H, o = i % H;
        float z = bias[o];
#pragma unroll
        for (int k = 0; k < IN; ++k) z += X[s * IN + k] * W1s[o * IN + k];
        if (s >= valid) z = 0.f;
        Z1[s * H + o] = z;
        H1[s * LDH + o] = __float2bfloat16_rn(silu(z));
    }
    __syncthreads();
    // layers 2 and 3 (128 -> 128) on the tensor cores: z = h . W^T, B(k=in, n=out) = W[n][k]
    float acc[8][4];
    const __nv_bfloat16 *Hs[2] = {H1, H2};
    const __nv_bfloat16 *Ws[2] = {W2s, W3s};
    float *Zs[2] = {Z2, Z3};
    __nv_bfloat16 *Ho[2] = {H2, H3};
#pragma unroll 1
    for (int l = 0; l < 2; ++l) {
        gemm_tile_x_h(Hs[l], LDH, 1, Ws[l], 1, LDH, acc);
#pragma unroll
        for (int j = 0; j < 8; ++j)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                int row, col;
                frag_coord(j, e, row, col);
                float z = acc[j][e] + bias[(l + 1) * H + col];
                if (row >= valid) z = 0.f;
                Zs[l][row * H + col] = z;
                Ho[l][row * LDH + col] = __float2bfloat16_rn(silu(z));
            }
        __syncthreads();
    }
    // layer 4 (128 -> 5), FP32 SIMT over BF16 activations
    for (int i = threadIdx.x; i < TILE * OUT; i += NT) {
        const int s = i / OUT, o = i % OUT;
        float v = bias[3 * H + o];
        for (int k = 0; k < H; ++k) v += __bfloat162float(H3[s * LDH + k]) * W4s[o * H + k];
        out[s * OUT + o] = v;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(NT) mlp_fwd_bwd_kernel(MlpDev m, TrainBatch b) {
    extern __shared__ __align__(16) unsigned char smem[];
    float *X = (float *)(smem + SmemLayout::X), *Y = (float *)(smem + SmemLayout::Y),
          *DO = (float *)(smem + SmemLayout::DO), *red = (float *)(smem + SmemLayout::RED);
    // this step's mini-batch: a slice of the shuffled epoch (perm is epoch-major)
    const long long step = b.step ? (*b.step - 1) : 0;
    const long long epoch = b.steps_per_epoch > 0 ? step / b.steps_per_epoch : 0;
    const long long batch0 = (b.steps_per_epoch > 0 ? (step % b.steps_per_epoch) : 0) * (long long)b.batch;
    const long long limit = b.steps_per_epoch > 0 ? (long long)b.n : (long long)b.batch;
    const int tiles = (b.batch + TILE - 1) / TILE;
    float *slot = m.partial + (size_t)blockIdx.x * kParamCount;
    float *gW4 = slot + OFF_W4, *gB4 = slot + OFF_B4, *gW1 = slot + OFF_W1, *gB1 = slot + OFF_B1;
    float *gW[2] = {slot + OFF_W3, slot + OFF_W2};
    float *gB[2] = {slot + OFF_B3, slot + OFF_B2};
    __nv_bfloat16 *W2s = (__nv_bfloat16 *)(smem + SmemLayout::W2);
    __nv_bfloat16 *W3s = (__nv_bfloat16 *)(smem + SmemLayout::W3);
    float *Z1 = (float *)(smem + SmemLayout::Z1), *Z2 = (float *)(smem + SmemLayout::Z2),
          *Z3 = (float *)(smem + SmemLayout::Z3);
    __nv_bfloat16 *H1 = (__nv_bfloat16 *)(smem + SmemLayout::H1), *H2 = (__nv_bfloat16 *)(smem + SmemLayout::H2),
                  *H3 = (__nv_bfloat16 *)(smem + SmemLayout::H3);
    float *W4s = (float *)(smem + SmemLayout::W4);
    // loss = mean over (batch, outputs) of the squared error in standardised units
    const float inv = 1.0f / ((float)b.batch * (float)OUT);
#pragma unroll 1
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const bool first = tile == (int)blockIdx.x;
        const long long base = batch0 + (long long)tile * TILE;
        int valid = (int)(limit - base);
        if (valid > TILE) valid = TILE;
        if (valid < 0) valid = 0;
        for (int i = threadIdx.x; i < TILE; i += NT) {
            const bool ok = i < valid;
            const long long idx = ok ? (b.perm ? (long long)b.perm[epoch * b.n + base + i] : base + i) : 0;
            for (int k = 0; k < IN; ++k) X[i * IN + k] = ok ? b.x[idx * IN + k] : 0.f;
            for (int k = 0; k < OUT; ++k) Y[i * OUT + k] = ok ? b.y[idx * OUT + k] : 0.f;
        }
        __syncthreads();
        float *out = DO;  // forward writes predictions here, backward turns them into dL/dout
        forward_tile(m, X, valid, smem, out);
        float lsum = 0.f;
        for (int i = threadIdx.x; i < TILE * OUT; i += NT) {
            const int s = i / OUT;
            float dlt = (s < valid) ? (out[i] - Y[i]) : 0.f;
            lsum += dlt * dlt;
            out[i] = 2.0f * dlt * inv;
        }
        block_reduce_acc(lsum * inv, red, &m.loss_part[blockIdx.x], first);
        // layer 4: dW4 = dout^T h3, db4 = sum dout  (FP32 SIMT)
        for (int i = threadIdx.x; i < OUT * H; i += NT) {
            const int o = i / H, k = i % H;
            float g = 0.f;
            for (int s = 0; s < TILE; ++s) g += DO[s * OUT + o] * __bfloat162float(H3[s * LDH + k]);
            slot_acc(&gW4[i], g, first);
        }
        if (threadIdx.x < OUT) {
            float g = 0.f;
            for (int s = 0; s < TILE; ++s) g += DO[s * OUT + threadIdx.x];
            slot_acc(&gB4[threadIdx.x], g, first);
        }
        __syncthreads();
        // delta3 = (dout W4) * silu'(z3) -> BF16 into H3's buffer
        for (int i = threadIdx.x; i < TILE * H; i += NT) {
            const int s = i / H, k = i % H;
            float v = 0.f;
#pragma unroll
            for (int o = 0; o < OUT; ++o) v += DO[s * OUT + o] * W4s[o * H + k];
            v *= silu_grad(Z3[s * H + k]);
            if (s >= valid) v = 0.f;
            H3[s * LDH + k] = __float2bfloat16_rn(v);
        }
        __syncthreads();
        // layers 3 and 2 on the tensor cores
        __nv_bfloat16 *Dl[2] = {H3, H2};   // delta of layer 3 (in H3), then of layer 2 (into H2)
        const __nv_bfloat16 *Hin[2] = {H2, H1};
        const __nv_bfloat16 *Wl[2] = {W3s, W2s};
        float *Zin[2] = {Z2, Z1};
#pragma unroll 1
        for (int l = 0; l < 2; ++l) {
            // bias gradient: column sums of delta
            for (int k = threadIdx.x; k < H; k += NT) {
                float g = 0.f;
                for (int s = 0; s < TILE; ++s) g += __bfloat162float(Dl[l][s * LDH + k]);
                slot_acc(&gB[l][k], g, first);
            }
            // weight gradient delta^T . h_in
            weight_grad(Dl[l], Hin[l], gW[l], first);
            __syncthreads();
            // input gradient: delta_in = (delta . W) * silu'(z_in), B(k=out, n=in) = W[k][n]
            float acc[8][4];
            gemm_tile_x_h(Dl[l], LDH, 1, Wl[l], LDH, 1, acc);
            __syncthreads();  // every warp has read delta_l before delta_in overwrites h_in (l = 1)
#pragma unroll
            for (int j = 0; j < 8; ++j)
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    int row, col;
                    frag_coord(j, e, row, col);
                    float v = acc[j][e] * silu_grad(Zin[l][row * H + col]);
                    if (row >= valid) v = 0.f;
                    if (l == 0) H2[row * LDH + col] = __float2bfloat16_rn(v);  // delta of layer 2
                    else Z1[row * H + col] = v;                                 // delta of layer 1 (FP32)
                }
            __syncthreads();
        }
        // layer 1: dW1 = delta1^T x, db1 = sum delta1  (FP32 SIMT; delta1 is in Z1)
        for (int i = threadIdx.x; i < H * IN; i += NT) {
            const int o = i / IN, k = i % IN;
            float g = 0.f;
            for (int s = 0; s < TILE; ++s) g += Z1[s * H + o] * X[s * IN + k];
            slot_acc(&gW1[i], g, first);
        }
        for (int o = threadIdx.x; o < H; o += NT) {
            float g = 0.f;
            for (int s = 0; s < TILE; ++s) g += Z1[s * H + o];
            slot_acc(&gB1[o], g, first);
        }
        __syncthreads();  // the next tile overwrites X, Y and the activations
    }
}

// step counter (first node of a captured step)
__global__ void mlp_step_begin_kernel(long long *step) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *step += 1;
}

// The step's gradient: the CTA slots summed in slot order (fixed, so bit-reproducible).
__device__ __forceinline__ float slot_sum(const MlpDev &m, int slots, int i) {
    float g = 0.f;
    for (int c = 0; c < slots; ++c) g += m.partial[(size_t)c * kParamCount + i];
    return g;
}
__device__ __forceinline__ void loss_sum(const MlpDev &m, int slots, float *loss) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        float l = 0.f;
        for (int c = 0; c < slots; ++c) l += m.loss_part[c];
        *loss = l;
    }
}

// gradient and loss of one batch, no update (the oracle check of the backward pass)
__global__ void mlp_reduce_kernel(MlpDev m, int slots, float *loss) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kParamCount; i += gridDim.x * blockDim.x)
        m.grad[i] = slot_sum(m, slots, i);
    loss_sum(m, slots, loss);
}

// BF16 copy of master parameter i (weights only; biases stay FP32)
__device__ __forceinline__ void refresh_bf16_at(const MlpDev &m, int i, float w) {
    const __nv_bfloat16 v = __float2bfloat16_rn(w);
    if (i < OFF_B1) m.w1b[i - OFF_W1] = v;
    else if (i >= OFF_W2 && i < OFF_B2) m.w2b[i - OFF_W2] = v;
    else if (i >= OFF_W3 && i < OFF_B3) m.w3b[i - OFF_W3] = v;
    else if (i >= OFF_W4 && i < OFF_B4) m.w4b[i - OFF_W4] = v;
}

// gradient (slot sums), Adam on the FP32 masters, BF16 refresh, the step's loss
__global__ void mlp_update_kernel(MlpDev m, int slots, const long long *step, AdamCfg c, float *loss) {
    const long long t = *step;
    // cosine decay of the learning rate over the run
    const double frac = c.total_steps > 0 ? fmin(1.0, (double)(t - 1) / (double)c.total_steps) : 0.0;
    const float lr = (float)(c.lr_min + 0.5 * (c.lr - c.lr_min) * (1.0 + cos(M_PI * frac)));
    const float bc1 = 1.0f - powf(c.beta1, (float)t), bc2 = 1.0f - powf(c.beta2, (float)t);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kParamCount; i += gridDim.x * blockDim.x) {
        const float g = slot_sum(m, slots, i);
        m.grad[i] = g;
        const float mm = c.beta1 * m.adam_m[i] + (1.0f - c.beta1) * g;
        const float vv = c.beta2 * m.adam_v[i] + (1.0f - c.beta2) * g * g;
        m.adam_m[i] = mm;
        m.adam_v[i] = vv;
        const float w = m.master[i] - lr * (mm / bc1) / (sqrtf(vv / bc2) + c.eps);
        m.master[i] = w;
        refresh_bf16_at(m, i, w);
    }
    loss_sum(m, slots, loss);
}

// BF16 copies of the weight matrices from the FP32 masters
__global__ void mlp_refresh_bf16_kernel(MlpDev m) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < H * H; i += gridDim.x * blockDim.x) {
        m.w2b[i] = __float2bfloat16_rn(m.master[OFF_W2 + i]);
        m.w3b[i] = __float2bfloat16_rn(m.master[OFF_W3 + i]);
        if (i < H * IN) m.w1b[i] = __float2bfloat16_rn(m.master[OFF_W1 + i]);
        if (i < OUT * H) m.w4b[i] = __float2bfloat16_rn(m.master[OFF_W4 + i]);
    }
}

// (T, mu, xi) in fm^-1 -> standardised network inputs
__global__ void mlp_prepare_inputs_kernel(Scaling sc, long long n, const double *T, const double *mu, const double *xi,
                                          float *x) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double v[3] = {T[i], mu[i], xi[i]};
        for (int k = 0; k < IN; ++k) x[i * IN + k] = (float)((v[k] - sc.in_shift[k]) / sc.in_scale[k]);
    }
}

__global__ void mlp_prepare_targets_kernel(Scaling sc, long long n, const double *xt, float *y) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        for (int k = 0; k < OUT; ++k) y[i * OUT + k] = (float)((xt[i * OUT + k] - sc.out_shift[k]) / sc.out_scale[k]);
}

// Forward pass over n points; de-standardised seeds [n x 5] (FP64) for the solver.
__global__ void __launch_bounds__(NT) mlp_infer_kernel(MlpDev m, Scaling sc, long long n, const double *T,
                                                        const double *mu, const double *xi, double *seeds) {
    extern __shared__ __align__(16) unsigned char smem[];
    float *X = (float *)(smem + SmemLayout::X), *out = (float *)(smem + SmemLayout::DO);
    for (long long tile = blockIdx.x; tile * TILE < n; tile += gridDim.x) {
        const long long base = tile * TILE;
        const int valid = (int)((n - base) < TILE ? (n - base) : TILE);
        for (int i = threadIdx.x; i < TILE; i += NT) {
            const bool ok = i < valid;
            const double v[3] = {ok ? T[base + i] : 0.0, ok ? mu[base + i] : 0.0, ok ? xi[base + i] : 0.0};
            for (int k = 0; k < IN; ++k) X[i * IN + k] = ok ? (float)((v[k] - sc.in_shift[k]) / sc.in_scale[k]) : 0.f;
        }
        __syncthreads();
        forward_tile(m, X, valid, smem, out);
        for (int i = threadIdx.x; i < valid * OUT; i += NT) {
            const int s = i / OUT, o = i % OUT;
            double v = (double)out[i] * sc.out_scale[o] + sc.out_shift[o];
            if (o < 2) {  // phi_u = phi_d: the network sees mu_u only, so its seed is isospin symmetric
                const double vu = (double)out[s * OUT + 0] * sc.out_scale[0] + sc.out_shift[0];
                const double vd = (double)out[s * OUT + 1] * sc.out_scale[1] + sc.out_shift[1];
                v = 0.5 * (vu + vd);
            }
            seeds[(base + s) * OUT + o] = v;
        }
        __syncthreads();
    }
}

}  // namespace mlp

// ---------------------------------------------------------------------------------------
// host side (called from the C ABI)
size_t mlp_smem_bytes() { return mlp::SmemLayout::TOTAL; }

cudaError_t mlp_setup_attributes() {
    cudaError_t e = cudaFuncSetAttribute(mlp::mlp_fwd_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)mlp::SmemLayout::TOTAL);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(mlp::mlp_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)mlp::SmemLayout::TOTAL);
}

int mlp_grad_slots(int batch) {
    const int tiles = (batch + mlp::TILE - 1) / mlp::TILE;
    return tiles < kMaxGradSlots ? tiles : kMaxGradSlots;
}

cudaError_t mlp_launch_step(const MlpDev &m, const TrainBatch &b, const AdamCfg &c, bool update, cudaStream_t s) {
    mlp::mlp_step_begin_kernel<<<1, 32, 0, s>>>(b.step);
    const int slots = mlp_grad_slots(b.batch);
    mlp::mlp_fwd_bwd_kernel<<<slots, mlp::NT, mlp::SmemLayout::TOTAL, s>>>(m, b);
    if (update)
        mlp::mlp_update_kernel<<<128, 256, 0, s>>>(m, slots, b.step, c, b.loss);
    else
        mlp::mlp_reduce_kernel<<<128, 256, 0, s>>>(m, slots, b.loss);
    return cudaGetLastError();
}

cudaError_t mlp_refresh_bf16(const MlpDev &m, cudaStream_t s) {
    mlp::mlp_refresh_bf16_kernel<<<64, 256, 0, s>>>(m);
    return cudaGetLastError();
}

cudaError_t mlp_prepare(const Scaling &sc, long long n, const double *T, const double *mu, const double *xi,
                        const double *targets, float *x, float *y, cudaStream_t s) {
    const int blocks = (int)((n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024);
    mlp::mlp_prepare_inputs_kernel<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(sc, n, T, mu, xi, x);
    if (targets) mlp::mlp_prepare_targets_kernel<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(sc, n, targets, y);
    return cudaGetLastError();
}

cudaError_t mlp_launch_infer(const MlpDev &m, const Scaling &sc, long long n, const double *T, const double *mu,
                             const double *xi, double *seeds, int sm_count, cudaStream_t s) {
    const long long tiles = (n + mlp::TILE - 1) / mlp::TILE;
    const int grid = (int)(tiles < (long long)sm_count * 2 ? tiles : (long long)sm_count * 2);
    mlp::mlp_infer_kernel<<<grid > 0 ? grid : 1, mlp::NT, mlp::SmemLayout::TOTAL, s>>>(m, sc, n, T, mu, xi, seeds);
    return cudaGetLastError();
}

}  // namespace pnjl
