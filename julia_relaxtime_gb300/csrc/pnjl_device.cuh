// pnjl_device.cuh -- device-side model of the PNJL grand potential for libpnjl_cuda.
//
// The integrand is restated from src/pnjl/core/Integrals.jl:178-259 (calculate_log_term,
// calculate_log_sum) in a branch-free form that needs one exponential and one reciprocal
// per node and flavour (plus one logarithm when Omega itself is wanted):
//
//   a = (mu - E)/T,  b = -(mu + E)/T = a - 2 mu/T,  t = exp(-|a|),  C = exp(-2 mu/T)  (mu >= 0)
//   f+ (the quark log argument)     = P(alpha, beta;   Phi, Phibar) / alpha^3
//   f- (the antiquark log argument) = P(alpha, C beta; Phibar, Phi) / alpha^3
//   P(alpha, beta; u, v) = alpha^3 + 3u alpha^2 beta + 3v alpha beta^2 + beta^3
//   (alpha, beta) = (1, t) for a <= 0 and (t, 1) for a > 0
//
// which is the reference's log-sum-exp rescaling (divide by e^{3a} when a > 0) applied to
// both factors.  mu < 0 uses the exact symmetry f+(mu, Phi, Phibar) = f-(-mu, Phibar, Phi).
// The reference's max(f, 1e-16) clamps (Integrals.jl:210,217,228,234) are kept: a clamped
// factor contributes the constant log(1e-16) (+3a in the rescaled branch) and no Phi
// derivatives, as ForwardDiff differentiates through max().
//
// Derivatives with respect to (M_f, Phi, Phibar) are analytic:
//   dL/da = 3 n+,  n+ = (Phi y + 2 Phibar y^2 + y^3)/f+  (the Polyakov quark distribution of
//   src/QuarkDistribution.jl:14-31), d2L/da2 = (3Phi y + 12Phibar y^2 + 9y^3)/f+ - 9 n+^2,
//   dE/dM = M/E, d2E/dM2 = p^2(1 + xi c^2)/E^3, and the mixed terms by the quotient rule.
//
// Node mesh: the reference's coefficient w_p (2 w_c) p^2/(2 pi)^2 (Integrals.jl:94) is kept
// separable, w = A[ip] * B[it] with A = w_p p^2/(2 pi)^2 and B = 2 w_c, and
// p^2 (1 + xi c^2) = p2[ip] * (1 + xi c2[it]); the tables are (p_num + t_num) entries.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "pnjl_f64.cuh"

namespace pnjl {

struct DevParams {
    double hbarc, Lambda, G, K, m_ud0, m_s0, T0, a0, a1, a2, b3, Nc, rho0;
};

// Sums of one pass over the node-flavour mesh (all in FP64 after the lane reduction).
// Index f = flavour (u, d, s); "P" = Phi, "Pb" = Phibar.
struct PassSums {
    double DM[3], DMM[3], DMP[3], DMPb[3], Nq[3], Na[3];
    double SL, SP, SPb, SPP, SPPb, SPbPb, SAN;
};

// Solver options on the device (see pnjl_solve_opts).
struct SolveOpts {
    int max_iter;
    double ftol, xtol, residual_norm_max, phi_tol, omega_tie_rtol;
    int trust_region_fallback, auto_multiseed_fallback;
    int verify_seeds;
    double verify_T_max_MeV, verify_max_step;
    const unsigned char *vmap;  // device copy of pnjl_solve_opts::verify_map, or null
    int vn[3];
    double vlo[3], vhi[3];
    // bounds of the fused kernel's waits on flags written by running warps of the same launch
    // (pnjl_set_wait_limits): polls of a listed slot's / queued job's ready flag, and of an
    // earlier seed's pending verdict; a wait that runs out gives up as documented there
    unsigned ready_polls, verdict_polls;
};

// Default wait bounds: 2^24 polls of 64 ns (about 1 s) for a ready flag, 2^20 polls of 128 ns
// for a pending verdict.
constexpr unsigned kReadyPollsDefault = 1u << 24;
constexpr unsigned kVerdictPollsDefault = 1u << 20;

// The reference's POLYAKOV_EPS (Integrals.jl:151) and log(POLYAKOV_EPS)
static constexpr double kPolyakovEps = 1e-16;
static constexpr double kLogPolyakovEps = -36.841361487904734;

// FP64 passes: in the rescaled branch (a > 0) t = exp(-min(a, kRescaleCapA)).  The antiquark
// variable C/t = exp(-(E + mu)/T) never exceeds t, so beyond the cap (t < 1.3e-100) every
// antiquark term is negligible against 1 in FP64, while t^3 (the rescaling of f-) stays a
// normal number: without the cap, t and C both underflow at T -> 0 and 0 * inf appears.
// The log term keeps the exact offset: ln f+ + ln f- = 3a + 3 min(a, cap) + ln(f+' f-').
static constexpr double kRescaleCapA = 230.0;

// Per-flavour constants of a pass.
template <typename R>
struct FlavourConst {
    R M, M2, mu, invT, C, C2, C3;
    R Pq, Pa;  // Phi on the quark side / antiquark side (swapped when mu < 0)
    // quark cubic Horner coefficients ((t + k2) t + k1) t + 1 for a <= 0 (index 0) and a > 0 (1)
    R k1_0, k2_0, k1_1, k2_1;
    // antiquark cubic ((e3 t + e2) t + e1) t + e0
    R e3_0, e2_0, e1_0, e0_0, e3_1, e2_1, e1_1, e0_1;
};

template <typename R>
__device__ __forceinline__ FlavourConst<R> make_flavour(double M, double mu, double T, double Phi, double Phib,
                                                      bool &swapped) {
    FlavourConst<R> fc;
    swapped = mu < 0.0;
    // the per-flavour constants are computed in the pass's own precision (an FP32 pass
    // spends no FP64 instructions here)
    const R mua = (R)(swapped ? -mu : mu);
    const R Pq = (R)(swapped ? Phib : Phi);
    const R Pa = (R)(swapped ? Phi : Phib);
    const R Tr = (R)T;
    R C;
    if constexpr (sizeof(R) == 4) C = __expf(-2.0f * mua / Tr);
    else C = exp(-2.0 * mua / Tr);
    const R C2 = C * C, C3 = C2 * C;
    fc.M = (R)M;
    fc.M2 = (R)M * (R)M;
    if constexpr (sizeof(R) == 8) fc.M2 = M * M;
    fc.mu = mua;
    fc.invT = R(1) / Tr;
    fc.C = C;
    fc.C2 = C2;
    fc.C3 = C3;
    fc.Pq = Pq;
    fc.Pa = Pa;
    fc.k1_0 = R(3) * Pq;
    fc.k2_0 = R(3) * Pa;
    fc.k1_1 = R(3) * Pa;
    fc.k2_1 = R(3) * Pq;
    fc.e3_0 = C3;
    fc.e2_0 = R(3) * Pq * C2;
    fc.e1_0 = R(3) * Pa * C;
    fc.e0_0 = R(1);
    fc.e3_1 = R(1);
    fc.e2_1 = R(3) * Pa * C;
    fc.e1_1 = R(3) * Pq * C2;
    fc.e0_1 = C3;
    return fc;
}

// Makes the per-flavour constants opaque register values for the node loop (see opaque()).
template <typename R>
__device__ __forceinline__ void opaque_flavour(FlavourConst<R> &fc) {
    opaque(fc.M); opaque(fc.M2); opaque(fc.mu); opaque(fc.invT); opaque(fc.C); opaque(fc.C2); opaque(fc.C3);
    opaque(fc.Pq); opaque(fc.Pa); opaque(fc.k1_0); opaque(fc.k2_0); opaque(fc.k1_1); opaque(fc.k2_1);
    opaque(fc.e3_0); opaque(fc.e2_0); opaque(fc.e1_0); opaque(fc.e0_0);
    opaque(fc.e3_1); opaque(fc.e2_1); opaque(fc.e1_1); opaque(fc.e0_1);
}

__device__ __forceinline__ double fast_exp(double x) { return exp(x); }
__device__ __forceinline__ float fast_exp(float x) { return __expf(x); }
__device__ __forceinline__ double fast_rcp(double x) { return 1.0 / x; }
// hardware approximation (MUFU, ~1 ulp): the FP32 passes' error budget is far above it
__device__ __forceinline__ float fast_rcp(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ double fast_rsqrt(double x) { return rsqrt(x); }
__device__ __forceinline__ float fast_rsqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ double fast_log(double x) { return log(x); }
__device__ __forceinline__ float fast_log(float x) { return __logf(x); }

// Accumulator: plain sum (FP64) or Kahan-compensated sum (FP32).
template <typename R, bool KAHAN>
struct Acc {
    R s;
    __device__ __forceinline__ void zero() { s = R(0); }
    __device__ __forceinline__ void add(R v) { s += v; }
    __device__ __forceinline__ double value() const { return (double)s; }
};
template <>
struct Acc<float, true> {
    float s, c;
    __device__ __forceinline__ void zero() { s = 0.f; c = 0.f; }
    __device__ __forceinline__ void add(float v) {
        float y = __fsub_rn(v, c);
        float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// Per-flavour accumulators of one lane over its share of the nodes.
template <typename R, bool KAHAN>
struct FlavourAcc {
    Acc<R, KAHAN> DM, Nq, Na, SL, Sq, Sa, SAN;
    // second derivatives (the Jacobian of the FP32 Newton steps): plain sums -- their lane
    // sums carry ~1e-6 relative error, far below what the steps and the refinement's
    // secant updates tolerate
    Acc<R, false> DMM, DMq, DMa, Sqq, Sqa, Saa;
    __device__ __forceinline__ void zero() {
        DM.zero(); DMM.zero(); DMq.zero(); DMa.zero(); Nq.zero(); Na.zero();
        SL.zero(); Sq.zero(); Sa.zero(); Sqq.zero(); Sqa.zero(); Saa.zero(); SAN.zero();
    }
};

// One node-flavour evaluation, accumulated with weight w.  q2 = p^2 (1 + xi c^2).
//   GRAD:   dD/dM_f, dD/dPhi, dD/dPhibar        (the residual F)
//   HESS:   the second derivatives              (the Jacobian J)
//   THERMO: ln f+ + ln f- (for Omega), sum w (a n+ + b n-) (entropy) and the per-flavour
//           sums of n+ and n- (rho_f and the number densities)
template <typename R, bool KAHAN, bool GRAD, bool HESS, bool THERMO>
__device__ __forceinline__ void node_flavour(const FlavourConst<R> &fc, R q2, R w, FlavourAcc<R, KAHAN> &acc) {
    const R E2 = q2 + fc.M2;
    const R rE = fast_rsqrt(E2);
    const R E = E2 * rE;
    const R mE = fc.M * rE;  // dE/dM
    const R a = (fc.mu - E) * fc.invT;
    const bool sig = a > R(0);
    // rescaling exponent of the a > 0 branch (capped in FP64, see kRescaleCapA)
    R ac = a;
    if constexpr (sizeof(R) == 8) ac = fmin(a, kRescaleCapA);
    const R t = fast_exp(sig ? -ac : a);
    const R t2 = t * t;
    const R t3 = t2 * t;
    const R k1 = sig ? fc.k1_1 : fc.k1_0;
    const R k2 = sig ? fc.k2_1 : fc.k2_0;
    const R fp = ((t + k2) * t + k1) * t + R(1);
    const R e3 = sig ? fc.e3_1 : fc.e3_0;
    const R e2 = sig ? fc.e2_1 : fc.e2_0;
    const R e1 = sig ? fc.e1_1 : fc.e1_0;
    const R e0 = sig ? fc.e0_1 : fc.e0_0;
    const R gm = ((e3 * t + e2) * t + e1) * t + e0;
    // clamps of the reference (max(f, 1e-16)); alpha^3 = t^3 when a > 0.  NaN is not
    // clamped (Julia's max propagates it).
    const R alpha3 = sig ? t3 : R(1);
    const bool clP = fp < R(kPolyakovEps);
    const bool clM = gm < R(kPolyakovEps) * alpha3;
    const R fpc = clP ? R(1) : fp;
    const R gmc = clM ? R(1) : gm;
    const R prod = fpc * gmc;
    const R Rr = fast_rcp(prod);
    const R ip = clP ? R(0) : gmc * Rr;
    const R im = clM ? R(0) : fpc * Rr;
    const R u1 = sig ? t2 : t;
    const R u2 = sig ? t : t2;
    const R u3 = sig ? R(1) : t3;
    const R r1 = u1 * ip, r2 = u2 * ip, r3 = u3 * ip;
    const R Cim = fc.C * im;
    const R s1 = u1 * Cim, s2 = fc.C * (u2 * Cim), s3 = fc.C2 * (u3 * Cim);
    const R Pq = fc.Pq, Pa = fc.Pa;
    const R np = clP ? (sig ? R(1) : R(0)) : (Pq * r1 + R(2) * Pa * r2 + r3);
    const R nm = clM ? R(0) : (Pa * s1 + R(2) * Pq * s2 + s3);
    const R invT = fc.invT;
    const R LE = R(-3) * (np + nm) * invT;
    if (GRAD) {
        acc.DM.add(w * (LE * mE));
        acc.Sq.add(w * (R(3) * (r1 + s2)));
        acc.Sa.add(w * (R(3) * (r2 + s1)));
    }
    if (THERMO) {
        acc.Nq.add(w * np);
        acc.Na.add(w * nm);
        const R b = a - R(2) * fc.mu * invT;
        acc.SAN.add(w * (a * np + b * nm));
        // ln f+ + ln f- = 6 max(a,0) + ln(fp gm); a clamped factor is replaced by the
        // reference's constant (log(1e-16), plus 3a in its rescaled quark branch)
        R L = (sig ? R(3) * (a + ac) : R(0)) + fast_log(prod);
        if (clP) L += R(kLogPolyakovEps);
        if (clM) L += R(kLogPolyakovEps) - (sig ? R(3) * ac : R(0));
        acc.SL.add(w * L);
    }
    if (HESS) {
        const R Laa = clP ? R(0) : (R(3) * Pq * r1 + R(12) * Pa * r2 + R(9) * r3 - R(9) * np * np);
        const R Lbb = clM ? R(0) : (R(3) * Pa * s1 + R(12) * Pq * s2 + R(9) * s3 - R(9) * nm * nm);
        const R LEE = (Laa + Lbb) * invT * invT;
        const R LMM = LEE * mE * mE + LE * (R(1) - mE * mE) * rE;
        const R LEq = -invT * (R(3) * r1 * (R(1) - R(3) * np) + R(3) * s2 * (R(2) - R(3) * nm));
        const R LEa = -invT * (R(3) * r2 * (R(2) - R(3) * np) + R(3) * s1 * (R(1) - R(3) * nm));
        acc.DMM.add(w * LMM);
        acc.DMq.add(w * (LEq * mE));
        acc.DMa.add(w * (LEa * mE));
        acc.Sqq.add(w * (R(-9) * (r1 * r1 + s2 * s2)));
        acc.Sqa.add(w * (R(-9) * (r1 * r2 + s1 * s2)));
        acc.Saa.add(w * (R(-9) * (r2 * r2 + s1 * s1)));
    }
}

}  // namespace pnjl
