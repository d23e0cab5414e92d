// pnjl_kdata.cu -- the K data of the relaxation-time chain per solved point: build_K_data
// (scripts/relaxtime/run_gap_transport_scan.jl:297-305).
//
// For every point, from the solved masses and Polyakov loops:
//   A_f  = 4 [ -int_0^Lambda p^2/E dp + sum_i w_i p_i^2/E_i (f+(E_i) + f-(E_i)) ]
//          (OneLoopIntegrals.jl:507-543; E = sqrt(p^2 + m_f^2), the PNJL distributions of
//          QuarkDistribution.jl:14-51), f = u and s, A_d = A_u;
//   G^f  = -N_c/(4 pi^2) m_f A_f                       (EffectiveCouplings.jl:56-60);
//   K0+-, K123+-, K4567+-, K8+-, K08+- and det K+-      (EffectiveCouplings.jl:112-115,242-279).
//
// One thread per point: the work is 2 x p_num node evaluations (128 at the reference's 64
// nodes) against 6 doubles read and up to 17 written, so a warp-per-point split would leave
// lanes idle; the node table sits in shared memory and every lane of a warp reads the same
// node (a broadcast).  Grid-stride loop, FP64 throughout (the chain that consumes these
// couplings is FP64 in the reference), sums in node order like the reference's loop.
#include "pnjl_kernels.h"

namespace pnjl {
namespace {

constexpr double kPi = 3.14159265358979323846;

__device__ __forceinline__ double const_term_A(double L, double m) {
    const double mp = m > 0.0 ? m : 0.0;
    if (mp < 1e-14) return L * L / 2.0;
    const double r = sqrt(L * L + mp * mp);
    return (L * r - mp * mp * log((L + r) / mp)) / 2.0;
}

// f+(E) + f-(E) with the reference's exp clamp to [1e-200, 1e200]
__device__ __forceinline__ double dist_pair(double E, double mu, double beta, double Phi, double Phib) {
    double y = exp(-(E - mu) * beta);
    y = fmin(fmax(y, 1e-200), 1e200);
    double z = exp(-(E + mu) * beta);
    z = fmin(fmax(z, 1e-200), 1e200);
    const double y2 = y * y, y3 = y2 * y, z2 = z * z, z3 = z2 * z;
    const double fp = (Phi * y + 2.0 * Phib * y2 + y3) / (1.0 + 3.0 * Phi * y + 3.0 * Phib * y2 + y3);
    const double fm = (Phib * z + 2.0 * Phi * z2 + z3) / (1.0 + 3.0 * Phib * z + 3.0 * Phi * z2 + z3);
    return fp + fm;
}

__device__ __forceinline__ double one_loop_A(const double *p, const double *w, int n, double L, double m, double mu,
                                             double T, double Phi, double Phib) {
    const double beta = 1.0 / T;
    double integral = -const_term_A(L, m);
    for (int i = 0; i < n; ++i) {
        const double E = sqrt(p[i] * p[i] + m * m);
        integral += w[i] * p[i] * p[i] / E * dist_pair(E, mu, beta, Phi, Phib);
    }
    return 4.0 * integral;
}

__device__ __forceinline__ void put(double *dst, int64_t i, double v) {
    if (dst) dst[i] = v;
}

__global__ void __launch_bounds__(256) kdata_kernel(KDataArgs a) {
    extern __shared__ double s_nodes[];  // p[p_num] | w[p_num]
    for (int i = threadIdx.x; i < a.p_num; i += blockDim.x) {
        s_nodes[i] = a.p[i];
        s_nodes[a.p_num + i] = a.w[i];
    }
    __syncthreads();
    const double *p = s_nodes, *w = s_nodes + a.p_num;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
        const double T = a.T[i], mu_u = a.mu_u[i], mu_s = a.mu_s[i];
        const double m_u = a.masses[3 * i], m_s = a.masses[3 * i + 2];
        const double Phi = a.x[5 * i + 3], Phib = a.x[5 * i + 4];
        const double Au = one_loop_A(p, w, a.p_num, a.Lambda, m_u, mu_u, T, Phi, Phib);
        const double As = one_loop_A(p, w, a.p_num, a.Lambda, m_s, mu_s, T, Phi, Phib);
        const double c = -3.0 / (4.0 * kPi * kPi);
        const double Gu = c * (m_u * Au), Gs = c * (m_s * As);
        const double G = a.G, K = a.K;
        const double t0 = (1.0 / 3.0) * K * (2.0 * Gu + Gs);
        const double t123 = 0.5 * K * Gs;
        const double t4567 = 0.5 * K * Gu;
        const double t8 = (1.0 / 6.0) * K * (4.0 * Gu - Gs);
        const double t08 = (1.0 / 6.0) * sqrt(2.0) * K * (Gu - Gs);
        const double K0p = G - t0, K0m = G + t0, K8p = G + t8, K8m = G - t8;
        const pnjl_kdata_soa &o = a.out;
        put(o.A_u, i, Au);
        put(o.A_d, i, Au);
        put(o.A_s, i, As);
        put(o.G_u, i, Gu);
        put(o.G_s, i, Gs);
        put(o.K0_plus, i, K0p);
        put(o.K0_minus, i, K0m);
        put(o.K123_plus, i, G + t123);
        put(o.K123_minus, i, G - t123);
        put(o.K4567_plus, i, G + t4567);
        put(o.K4567_minus, i, G - t4567);
        put(o.K8_plus, i, K8p);
        put(o.K8_minus, i, K8m);
        put(o.K08_plus, i, t08);
        put(o.K08_minus, i, -t08);
        put(o.det_K_plus, i, K0p * K8p - t08 * t08);
        put(o.det_K_minus, i, K0m * K8m - t08 * t08);
    }
}

}  // namespace

cudaError_t launch_kdata(const KDataArgs &a, int sm_count, cudaStream_t s) {
    if (a.n <= 0) return cudaSuccess;
    const int64_t blocks = (a.n + 255) / 256;
    const int64_t cap = (int64_t)sm_count * 8;
    const int grid = (int)(blocks < cap ? blocks : cap);
    kdata_kernel<<<grid, 256, 2 * (size_t)a.p_num * sizeof(double), s>>>(a);
    return cudaGetLastError();
}

}  // namespace pnjl
