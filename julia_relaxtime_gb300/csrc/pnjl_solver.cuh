// pnjl_solver.cuh -- passes, assembly and the NLsolve-style Newton / trust-region drivers
// that run inside one lane group (G lanes cooperate on one point; G = 32 is one warp).
//
// Reference semantics restated here (w5851/Julia_RelaxTime):
//   Omega and its parts ....... src/pnjl/core/Thermodynamics.jl:81-206, Integrals.jl:123-145
//   F = grad_x P, J = dF/dx .... src/pnjl/solver/Conditions.jl:72-86 (ForwardDiff, here analytic)
//   Newton ..................... ImplicitSolver.jl:112 -> NLsolve 4.5.1 :newton, static line
//                                search: full step, converged iff ||F||_inf < ftol or
//                                ||x - x_prev||_inf < xtol, singular J -> LM direction
//   trust region ............... ImplicitSolver.jl:144 -> NLsolve :trust_region (dogleg,
//                                autoscale, factor 1, eta 1e-4)
//   physicality, candidate choice ImplicitSolver.jl:50-101
//   thermo ..................... Thermodynamics.jl:215-244 (rho = dP/dmu, s = dP/dT analytic)
#pragma once

#include "pnjl_device.cuh"
#include "pnjl_f64.cuh"
#include "pnjl_ff.cuh"

namespace pnjl {

struct PointIn {
    double T, mu[3], xi;
};

// Result of one evaluation at a state x (FP64 assembly).
struct Eval {
    double F[5];   // grad_x P = -grad_x Omega
    double J[25];  // Hessian_x P, row-major
    double omega;
    double dOdT;   // dOmega/dT at fixed x, mu
    double rho[3];
    double nq[3], naq[3];
};

// Separable node tables (see pnjl_device.cuh): p2[ip], A[ip] over p; c2[it], B[it] over t.
struct NodeView {
    const double *p2, *A, *c2, *B;
    const float *p2f, *Af, *c2f, *Bf;
    const float *p2l, *Al, *c2l, *Bl;  // float-float low parts (null when not staged)
    const float *expt;                 // float-float exp tables (null when not staged)
    const double *exp64;               // 2^(j/256) table of exp_nonpos (null when not staged)
    int p_num, t_num;
};

__device__ __forceinline__ void masses(const DevParams &P, const double *x, double *M) {
    M[0] = P.m_ud0 - 4.0 * P.G * x[0] + 2.0 * P.K * x[1] * x[2];
    M[1] = P.m_ud0 - 4.0 * P.G * x[1] + 2.0 * P.K * x[0] * x[2];
    M[2] = P.m_s0 - 4.0 * P.G * x[2] + 2.0 * P.K * x[0] * x[1];
}

template <int G>
__device__ __forceinline__ unsigned group_mask(int lane) {
    if constexpr (G == 32) {
        return 0xffffffffu;
    } else {
        const unsigned base = (unsigned)(lane & ~(G - 1));
        return ((1u << G) - 1u) << base;
    }
}

// XOR butterfly: a + b == b + a bitwise, so every lane of the group ends with the
// identical sum and the group's control flow stays uniform.
template <int G>
__device__ __forceinline__ double group_sum(double v, unsigned mask) {
#pragma unroll
    for (int m = G >> 1; m > 0; m >>= 1) v += __shfl_xor_sync(mask, v, m);
    return v;
}

// Float-float XOR butterfly: TwoSum gives the exact rounding error of h_a + h_b, which does
// not depend on the operand order, so every lane again ends with identical bits.
template <int G>
__device__ __forceinline__ void group_sum_ff(float &h, float &l, unsigned mask) {
#pragma unroll
    for (int m = G >> 1; m > 0; m >>= 1) {
        const float bh = __shfl_xor_sync(mask, h, m);
        const float bl = __shfl_xor_sync(mask, l, m);
        const float sum = __fadd_rn(h, bh);
        const float hp = __fsub_rn(sum, bh);
        const float bp = __fsub_rn(sum, hp);
        const float err = __fadd_rn(__fsub_rn(h, hp), __fsub_rn(bh, bp));
        l = __fadd_rn(__fadd_rn(l, bl), err);
        h = sum;
    }
}

// Vacuum term -2 Nc sum_f I(|M_f| + 1e-12) and its first two derivatives in M_f
// (Integrals.jl:123-145), FP64, lane-parallel: lane f of the group computes flavour f and the
// results are broadcast, so the three evaluations cost one instruction stream.
template <int G>
__device__ __forceinline__ void vacuum_terms(const DevParams &P, const double *M, int gl, unsigned mask, int leader,
                                             double &V, double *V1, double *V2) {
    const int f = (G >= 4) ? (gl % 3) : 0;
    const double L = P.Lambda;
    const double inv4pi2 = 1.0 / (4.0 * M_PI * M_PI);
    auto one = [&](double m, double &I, double &I1, double &I2) {
        const double sgn = signbit(m) ? -1.0 : 1.0;
        const double ms = fabs(m) + 1e-12;
        const double ms2 = ms * ms;
        const double Sq = sqrt(L * L + ms2);
        const double lgv = log((L + Sq) / ms);
        I = (L * Sq * (2.0 * L * L + ms2) - ms2 * ms2 * lgv) * (0.25 * inv4pi2);
        I1 = -2.0 * P.Nc * ((L * ms * Sq - ms2 * ms * lgv) * inv4pi2) * sgn;
        I2 = -2.0 * P.Nc * ((L * Sq + 2.0 * L * ms2 / Sq - 3.0 * ms2 * lgv) * inv4pi2);
    };
    if (G >= 4) {
        const double mf = f == 0 ? M[0] : (f == 1 ? M[1] : M[2]);
        double I, I1, I2;
        one(mf, I, I1, I2);
        double Is[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            Is[k] = __shfl_sync(mask, I, leader + k);
            V1[k] = __shfl_sync(mask, I1, leader + k);
            V2[k] = __shfl_sync(mask, I2, leader + k);
        }
        V = ((Is[0] + Is[1]) + Is[2]) * (-2.0 * P.Nc);
    } else {
        double Is[3];
        for (int k = 0; k < 3; ++k) one(M[k], Is[k], V1[k], V2[k]);
        V = ((Is[0] + Is[1]) + Is[2]) * (-2.0 * P.Nc);
    }
}

// Per-pass sums of node_pass, per lane before the group reduction.  FP64 passes keep
// doubles.  FP32 (Kahan) passes keep each sum as a float pair (h, l) -- a flavour's Kahan
// accumulator (s, c) enters as (s, -c) -- and reduce the pairs over the lanes by TwoSum
// butterflies, so that only the final value of each sum is converted to FP64: the FP64 pipe,
// the scarcest on the GB300, sees 3 instructions per sum instead of about 10.
template <typename R, bool KAHAN>
struct PassAcc {
    double v[25];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int i = 0; i < 25; ++i) v[i] = 0.0;
    }
    __device__ __forceinline__ void set(int i, const Acc<R, KAHAN> &a) { v[i] = a.value(); }
    __device__ __forceinline__ void add(int i, bool twice, const Acc<R, KAHAN> &a) {
        v[i] += (twice ? 2.0 : 1.0) * a.value();
    }
    template <int G>
    __device__ __forceinline__ double reduce(int i, unsigned mask) { return group_sum<G>(v[i], mask); }
};
template <>
struct PassAcc<float, true> {
    float h[25], l[25];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int i = 0; i < 25; ++i) h[i] = l[i] = 0.0f;
    }
    __device__ __forceinline__ void set(int i, const Acc<float, true> &a) { h[i] = a.s; l[i] = -a.c; }
    __device__ __forceinline__ void set(int i, const Acc<float, false> &a) { h[i] = a.s; l[i] = 0.0f; }
    __device__ __forceinline__ void add(int i, bool twice, const Acc<float, false> &a) {
        Acc<float, true> k;
        k.s = a.s;
        k.c = 0.0f;
        add(i, twice, k);
    }
    __device__ __forceinline__ void add(int i, bool twice, const Acc<float, true> &a) {
        const float m = twice ? 2.0f : 1.0f;  // exact scaling
        const float bh = m * a.s, bl = -m * a.c;
        const float sum = __fadd_rn(h[i], bh);
        const float hp = __fsub_rn(sum, bh);
        const float err = __fadd_rn(__fsub_rn(h[i], hp), __fsub_rn(bh, __fsub_rn(sum, hp)));
        l[i] = __fadd_rn(__fadd_rn(l[i], bl), err);
        h[i] = sum;
    }
    template <int G>
    __device__ __forceinline__ double reduce(int i, unsigned mask) {
        float hh = h[i], ll = l[i];
        group_sum_ff<G>(hh, ll, mask);
        return (double)hh + (double)ll;
    }
};

// One pass over the node-flavour mesh at state x; lane `gl` of a group of G lanes takes
// the flattened nodes k = gl, gl+G, ... (k = ip + p_num*it).  Returns the group-reduced
// sums (identical in every lane of the group); entries a pass does not compute are 0.
template <typename R, bool KAHAN, bool GRAD, bool HESS, bool THERMO, int G>
__device__ void node_pass(const NodeView &nv, const PointIn &pt, const double *x, const double *M, int gl,
                          unsigned mask, PassSums &S, int64_t &evals) {
    constexpr int NS = 25;
    PassAcc<R, KAHAN> acc;
    acc.zero();
    const bool dedup = (M[1] == M[0]) && (pt.mu[1] == pt.mu[0]);
    const R *p2, *A, *c2, *B;
    if constexpr (sizeof(R) == 8) { p2 = (const R *)nv.p2; A = (const R *)nv.A; c2 = (const R *)nv.c2; B = (const R *)nv.B; }
    else { p2 = (const R *)nv.p2f; A = (const R *)nv.Af; c2 = (const R *)nv.c2f; B = (const R *)nv.Bf; }
    const int pn = nv.p_num, n = nv.p_num * nv.t_num;
    const R xi = (R)pt.xi;
#pragma unroll 1
    for (int f = 0; f < 3; ++f) {
        if (f == 1 && dedup) continue;
        bool sw;
        FlavourConst<R> fc = make_flavour<R>(M[f], pt.mu[f], pt.T, x[3], x[4], sw);
        opaque_flavour(fc);
        FlavourAcc<R, KAHAN> fa;
        fa.zero();
        int ip = gl, it = 0;
        while (ip >= pn) { ip -= pn; ++it; }
        R sxi = R(1), bw = R(0);
        if (it < nv.t_num) { sxi = xi * c2[it] + R(1); bw = B[it]; }
#pragma unroll 1
        for (int k = gl; k < n; k += G) {
            const R pp = p2[ip];
            node_flavour<R, KAHAN, GRAD, HESS, THERMO>(fc, pp * sxi, A[ip] * bw, fa);
            ip += G;
            if (ip >= pn) {
                do { ip -= pn; ++it; } while (ip >= pn);
                if (it < nv.t_num) { sxi = xi * c2[it] + R(1); bw = B[it]; }
            }
        }
        const bool two = (f == 0 && dedup);
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            if (j == 1 && !two) break;
            const int ff = j == 0 ? f : 1;
            if (GRAD) acc.set(0 + ff, fa.DM);
            if (HESS) {
                acc.set(3 + ff, fa.DMM);
                acc.set(6 + ff, sw ? fa.DMa : fa.DMq);
                acc.set(9 + ff, sw ? fa.DMq : fa.DMa);
            }
            if (THERMO) {
                acc.set(12 + ff, sw ? fa.Na : fa.Nq);
                acc.set(15 + ff, sw ? fa.Nq : fa.Na);
            }
        }
        if (GRAD) {
            acc.add(19, two, sw ? fa.Sa : fa.Sq);
            acc.add(20, two, sw ? fa.Sq : fa.Sa);
        }
        if (HESS) {
            acc.add(21, two, sw ? fa.Saa : fa.Sqq);
            acc.add(22, two, fa.Sqa);
            acc.add(23, two, sw ? fa.Sqq : fa.Saa);
        }
        if (THERMO) {
            acc.add(18, two, fa.SL);
            acc.add(24, two, fa.SAN);
        }
        if (gl == 0) evals += (int64_t)n;
    }
    double r[NS];
#pragma unroll
    for (int i = 0; i < NS; ++i) {
        const bool used = (i < 3 || i == 19 || i == 20) ? GRAD
                          : (i < 12 || (i >= 21 && i <= 23)) ? HESS : THERMO;
        r[i] = used ? acc.template reduce<G>(i, mask) : 0.0;
    }
    for (int f = 0; f < 3; ++f) {
        S.DM[f] = r[0 + f]; S.DMM[f] = r[3 + f]; S.DMP[f] = r[6 + f]; S.DMPb[f] = r[9 + f];
        S.Nq[f] = r[12 + f]; S.Na[f] = r[15 + f];
    }
    S.SL = r[18]; S.SP = r[19]; S.SPb = r[20]; S.SPP = r[21]; S.SPPb = r[22]; S.SPbPb = r[23];
    S.SAN = r[24];
}

// FP32 Newton pass of the mixed solver: the residual and Jacobian sums of
// node_pass<float, KAHAN, GRAD, HESS> in a form with fewer instructions per node-flavour --
// it runs on most of the solver's node evaluations.  Per node, with u, r_k = u_k/f+,
// s_k = C^(k-1) u_k/f-, n+ and n- as in node_pass_cert, and m = M/E:
//   D   = sum w (n+ + n-) m                       -> S.DM  = -3/T D
//   Q   = sum w (r1 + s2),  A = sum w (r2 + s1)   -> S.SP, S.SPb = 3 Q, 3 A (sides by mu's sign)
//   H1  = sum w (L++ + L--) m^2,  H2 = sum w (n+ + n-)(1 - m^2)/E
//                                                 -> S.DMM = H1/T^2 - 3 H2/T
//       with L++ = 3 n+ + 6 (Phibar r2 + r3) - 9 n+^2, L-- = 3 n- + 6 (Phi s2 + s3) - 9 n-^2
//   Pq  = sum w m (r1 (1 - 3n+) + s2 (2 - 3n-)), Pa = sum w m (r2 (2 - 3n+) + s1 (1 - 3n-))
//                                                 -> S.DMP, S.DMPb = -3/T Pq, -3/T Pa
//   Sqq, Sqa, Saa = sum w (r1^2 + s2^2), (r1 r2 + s1 s2), (r2^2 + s1^2) -> times -9
// (the second derivatives of node_flavour regrouped; a clamped factor contributes no Phi
// terms).  The three residual sums are Kahan-compensated, the Jacobian's plain; all are
// reduced over the lanes as float pairs.
template <int G>
__device__ void node_pass_newton32(const NodeView &nv, const PointIn &pt, const double *x, const double *M, int gl,
                                   unsigned mask, PassSums &S, int64_t &evals) {
    const bool dedup = (M[1] == M[0]) && (pt.mu[1] == pt.mu[0]);
    const float *p2 = nv.p2f, *A = nv.Af, *c2 = nv.c2f, *B = nv.Bf;
    const int pn = nv.p_num, n = nv.p_num * nv.t_num;
    const float xi = (float)pt.xi;
    // per-flavour results (lane partials) as float pairs: 0 D, 1 H1, 2 H2, 3 Pq, 4 Pa
    float fh[3][5], fl[3][5];
    // side sums over the flavours: 0 Q-side (Phi), 1 A-side (Phibar), 2 Sqq-side, 3 Sqa, 4 Saa-side
    float sh[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, sl[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    auto pair_add = [](float &h, float &l, float bh, float bl) {
        const float sum = __fadd_rn(h, bh);
        const float hp = __fsub_rn(sum, bh);
        const float err = __fadd_rn(__fsub_rn(h, hp), __fsub_rn(bh, __fsub_rn(sum, hp)));
        l = __fadd_rn(__fadd_rn(l, bl), err);
        h = sum;
    };
    for (int f = 0; f < 3; ++f)
        for (int k = 0; k < 5; ++k) fh[f][k] = fl[f][k] = 0.0f;
#pragma unroll 1
    for (int f = 0; f < 3; ++f) {
        if (f == 1 && dedup) continue;
        bool sw;
        FlavourConst<float> fc = make_flavour<float>(M[f], pt.mu[f], pt.T, x[3], x[4], sw);
        float muT = fc.mu * fc.invT, Pa2 = 2.0f * fc.Pa, Pq2 = 2.0f * fc.Pq;
        opaque_flavour(fc);
        opaque(muT); opaque(Pa2); opaque(Pq2);
        Acc<float, true> aD, aQ, aA;
        aD.zero(); aQ.zero(); aA.zero();
        float H1 = 0.f, H2 = 0.f, PQ = 0.f, PA = 0.f, Sqq = 0.f, Sqa = 0.f, Saa = 0.f;
        int ip = gl, it = 0;
        while (ip >= pn) { ip -= pn; ++it; }
        float sxi = 1.0f, bw = 0.0f;
        if (it < nv.t_num) { sxi = __fmaf_rn(xi, c2[it], 1.0f); bw = B[it]; }
#pragma unroll 1
        for (int k = gl; k < n; k += G) {
            const float w = A[ip] * bw;
            const float E2 = __fmaf_rn(p2[ip], sxi, fc.M2);
            const float rE = rsqrtf(E2);
            const float E = E2 * rE, m = fc.M * rE;
            const float a = __fmaf_rn(-E, fc.invT, muT);
            const bool sig = a > 0.0f;
            const float t = __expf(sig ? -a : a);
            const float t2 = t * t, t3 = t2 * t;
            const float fp = __fmaf_rn(__fmaf_rn(t + (sig ? fc.k2_1 : fc.k2_0), t, sig ? fc.k1_1 : fc.k1_0), t, 1.0f);
            const float gm = __fmaf_rn(__fmaf_rn(__fmaf_rn(sig ? 1.0f : fc.e3_0, t, sig ? fc.e2_1 : fc.e2_0), t,
                                                 sig ? fc.e1_1 : fc.e1_0), t, sig ? fc.e0_1 : 1.0f);
            const bool clP = fp < 1e-16f;
            const bool clM = gm < 1e-16f * (sig ? t3 : 1.0f);
            const float ipv = clP ? 0.0f : fast_rcp(fp);
            const float im = clM ? 0.0f : fast_rcp(gm);
            const float u1 = sig ? t2 : t, u2 = sig ? t : t2, u3 = sig ? 1.0f : t3;
            const float r1 = u1 * ipv, r2 = u2 * ipv, r3 = u3 * ipv;
            const float C1 = fc.C * im, C2i = fc.C * C1, C3i = fc.C * C2i;
            const float s1 = u1 * C1, s2 = u2 * C2i, s3 = u3 * C3i;
            const float np = clP ? (sig ? 1.0f : 0.0f) : __fmaf_rn(fc.Pq, r1, __fmaf_rn(Pa2, r2, r3));
            const float nm = clM ? 0.0f : __fmaf_rn(fc.Pa, s1, __fmaf_rn(Pq2, s2, s3));
            const float npnm = np + nm;
            aD.add(w * (npnm * m));
            aQ.add(w * (r1 + s2));
            aA.add(w * (r2 + s1));
            const float Lpp = clP ? 0.0f : __fmaf_rn(-9.0f * np, np, __fmaf_rn(6.0f, __fmaf_rn(fc.Pa, r2, r3), 3.0f * np));
            const float Lmm = clM ? 0.0f : __fmaf_rn(-9.0f * nm, nm, __fmaf_rn(6.0f, __fmaf_rn(fc.Pq, s2, s3), 3.0f * nm));
            const float m2 = m * m;
            const float wm = w * m;
            H1 = __fmaf_rn(wm * m, Lpp + Lmm, H1);
            H2 = __fmaf_rn(w * npnm, (1.0f - m2) * rE, H2);
            const float np3 = 3.0f * np, nm3 = 3.0f * nm;
            PQ = __fmaf_rn(wm, __fmaf_rn(r1, 1.0f - np3, s2 * (2.0f - nm3)), PQ);
            PA = __fmaf_rn(wm, __fmaf_rn(r2, 2.0f - np3, s1 * (1.0f - nm3)), PA);
            Sqq = __fmaf_rn(w, __fmaf_rn(r1, r1, s2 * s2), Sqq);
            Sqa = __fmaf_rn(w, __fmaf_rn(r1, r2, s1 * s2), Sqa);
            Saa = __fmaf_rn(w, __fmaf_rn(r2, r2, s1 * s1), Saa);
            ip += G;
            if (ip >= pn) {
                do { ip -= pn; ++it; } while (ip >= pn);
                if (it < nv.t_num) { sxi = __fmaf_rn(xi, c2[it], 1.0f); bw = B[it]; }
            }
        }
        const bool two = (f == 0 && dedup);
        const float mult = two ? 2.0f : 1.0f;  // exact scaling
        fh[f][0] = aD.s; fl[f][0] = -aD.c;
        fh[f][1] = H1; fh[f][2] = H2;
        fh[f][3] = sw ? PA : PQ;
        fh[f][4] = sw ? PQ : PA;
        const Acc<float, true> &qq = sw ? aA : aQ, &aa = sw ? aQ : aA;
        pair_add(sh[0], sl[0], mult * qq.s, -mult * qq.c);
        pair_add(sh[1], sl[1], mult * aa.s, -mult * aa.c);
        pair_add(sh[2], sl[2], mult * (sw ? Saa : Sqq), 0.0f);
        pair_add(sh[3], sl[3], mult * Sqa, 0.0f);
        pair_add(sh[4], sl[4], mult * (sw ? Sqq : Saa), 0.0f);
        if (two)
            for (int k = 0; k < 5; ++k) { fh[1][k] = fh[0][k]; fl[1][k] = fl[0][k]; }
        if (gl == 0) evals += (int64_t)n;
    }
    double r[3][5];
    for (int f = 0; f < 3; ++f)
        for (int k = 0; k < 5; ++k) {
            float hh = fh[f][k], ll = fl[f][k];
            group_sum_ff<G>(hh, ll, mask);
            r[f][k] = (double)hh + (double)ll;
        }
    double q[5];
    for (int k = 0; k < 5; ++k) {
        float hh = sh[k], ll = sl[k];
        group_sum_ff<G>(hh, ll, mask);
        q[k] = (double)hh + (double)ll;
    }
    const double iT = 1.0 / pt.T;
    for (int f = 0; f < 3; ++f) {
        S.DM[f] = -3.0 * iT * r[f][0];
        S.DMM[f] = iT * iT * r[f][1] - 3.0 * iT * r[f][2];
        S.DMP[f] = -3.0 * iT * r[f][3];
        S.DMPb[f] = -3.0 * iT * r[f][4];
        S.Nq[f] = S.Na[f] = 0.0;
    }
    S.SP = 3.0 * q[0];
    S.SPb = 3.0 * q[1];
    S.SPP = -9.0 * q[2];
    S.SPPb = -9.0 * q[3];
    S.SPbPb = -9.0 * q[4];
    S.SL = S.SAN = 0.0;
}

// FP64 residual pass of the mixed solve's certification: the sums S.DM, S.SP, S.SPb of
// node_pass<double, GRAD only> from the same integrand in FP64, arranged for the FP64 pipe
// (52 FP64 instructions per node-flavour, measured): exp, 1/x and 1/sqrt from pnjl_f64.cuh,
// Horner forms in FMAs, integer selects and clamp compares, opaque loop invariants, and the
// per-flavour factors -3 M/T (dOmega/dM, with dE/dM = M/E), 3 (dOmega/dPhi) and C, C^2 (the
// Phi derivatives' f- terms, summed without them) applied once to the lane sums instead of
// per node.  With r_k = u_k / f+ and s_k = C^(k-1) u_k / f- (u = (t, t^2, t^3)
// for a <= 0, (t^2, t, 1) for a > 0) the Polyakov distributions are
//   n+ = (Phi u1 + 2 Phibar u2 + u3) / f+,   n- = C (Phibar u1 + 2 Phi C u2 + C^2 u3) / f-
// and the Phi / Phibar derivatives take r1 + s2 and r2 + s1 (quark / antiquark sides
// swapped for mu < 0).  Requires the staged FP64 exp table (nv.exp64).
template <int G>
__device__ void node_pass_cert(const NodeView &nv, const PointIn &pt, const double *x, const double *M, int gl,
                               unsigned mask, PassSums &S, int64_t &evals) {
    const bool dedup = (M[1] == M[0]) && (pt.mu[1] == pt.mu[0]);
    const double *p2 = nv.p2, *A = nv.A, *c2 = nv.c2, *B = nv.B, *tab = nv.exp64;
    const int pn = nv.p_num, n = nv.p_num * nv.t_num;
    const double xi = pt.xi;
    const unsigned long long cap = (unsigned long long)__double_as_longlong(-kRescaleCapA);
    const long long epsb = __double_as_longlong(kPolyakovEps);
    double DM[3] = {0.0, 0.0, 0.0}, SP = 0.0, SPb = 0.0;
#pragma unroll 1
    for (int f = 0; f < 3; ++f) {
        if (f == 1 && dedup) continue;
        bool sw;
        const FlavourConst<double> fc = make_flavour<double>(M[f], pt.mu[f], pt.T, x[3], x[4], sw);
        double M2 = fc.M2, invT = fc.invT, muT = fc.mu * fc.invT, C = fc.C, C2 = fc.C2;
        double Pq = fc.Pq, Pa = fc.Pa, Pa2 = 2.0 * fc.Pa, Pq2C = 2.0 * fc.Pq * fc.C;
        double k1_0 = fc.k1_0, k2_0 = fc.k2_0, k1_1 = fc.k1_1, k2_1 = fc.k2_1;
        double e3_0 = fc.e3_0, e2_0 = fc.e2_0, e1_0 = fc.e1_0, e2_1 = fc.e2_1, e1_1 = fc.e1_1, e0_1 = fc.e0_1;
        opaque(M2); opaque(invT); opaque(muT); opaque(C); opaque(C2);
        opaque(Pq); opaque(Pa); opaque(Pa2); opaque(Pq2C);
        opaque(k1_0); opaque(k2_0); opaque(k1_1); opaque(k2_1);
        opaque(e3_0); opaque(e2_0); opaque(e1_0); opaque(e2_1); opaque(e1_1); opaque(e0_1);
        // sq = s1 + C^2 s4 and sa = s2 + C s3: the sums of w/f+ u_k and w/f- u_k
        double dm = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0, s4 = 0.0;
        int ip = gl, it = 0;
        while (ip >= pn) { ip -= pn; ++it; }
        double sxi = 1.0, bw = 0.0;
        if (it < nv.t_num) { sxi = fma(xi, c2[it], 1.0); bw = B[it]; }
#pragma unroll 1
        for (int k = gl; k < n; k += G) {
            const double w = A[ip] * bw;
            const double E2 = fma(p2[ip], sxi, M2);
            const double rE = rsqrt_normal(E2);
            const double a = fma(-E2 * rE, invT, muT);  // (mu - E)/T
            // a > 0, and -min(a, kRescaleCapA) or a, from the bit patterns (integer pipe):
            // among negative doubles the larger pattern is the larger magnitude
            const long long ab = __double_as_longlong(a);
            const bool sig = ab > 0;
            const unsigned long long nb = (unsigned long long)ab | 0x8000000000000000ull;
            const double t = exp_nonpos(__longlong_as_double((long long)(sig && nb > cap ? cap : nb)), tab);
            const double t2 = t * t, t3 = t2 * t;
            const double fp = fma(fma(t + dsel(sig, k2_1, k2_0), t, dsel(sig, k1_1, k1_0)), t, 1.0);
            const double gm =
                fma(fma(fma(dsel(sig, 1.0, e3_0), t, dsel(sig, e2_1, e2_0)), t, dsel(sig, e1_1, e1_0)), t, dsel(sig, e0_1, 1.0));
            // the reference's max(f, 1e-16) clamps, compared as bit patterns on the integer pipe
            // (the same order as the doubles' for all but -0.0 and negative NaNs, which f+ and
            // f- -- polynomials in t in [0, 1] with finite coefficients -- never take)
            const bool clP = __double_as_longlong(fp) < epsb;
            const bool clM = __double_as_longlong(gm) < __double_as_longlong(kPolyakovEps * dsel(sig, t3, 1.0));
            const double fpc = dsel(clP, 1.0, fp), gmc = dsel(clM, 1.0, gm);
            const double Rr = rcp_normal(fpc * gmc);
            const double ipv = dsel(clP, 0.0, gmc * Rr);  // 1/f+
            const double im = dsel(clM, 0.0, fpc * Rr);   // 1/f-
            const double u1 = dsel(sig, t2, t), u2 = dsel(sig, t, t2), u3 = dsel(sig, 1.0, t3);
            const double Cim = C * im;
            const double np = dsel(clP, dsel(sig, 1.0, 0.0), ipv * fma(Pq, u1, fma(Pa2, u2, u3)));
            const double nm = dsel(clM, 0.0, Cim * fma(Pa, u1, fma(Pq2C, u2, C2 * u3)));
            dm = fma(w, (np + nm) * rE, dm);
            const double wp = w * ipv, wm = w * im;
            s1 = fma(wp, u1, s1);
            s2 = fma(wp, u2, s2);
            s3 = fma(wm, u1, s3);
            s4 = fma(wm, u2, s4);
            ip += G;
            if (ip >= pn) {
                do { ip -= pn; ++it; } while (ip >= pn);
                if (it < nv.t_num) { sxi = fma(xi, c2[it], 1.0); bw = B[it]; }
            }
        }
        const double mult = (f == 0 && dedup) ? 2.0 : 1.0;
        const double sq = fma(fc.C2, s4, s1), sa = fma(fc.C, s3, s2);
        DM[f] = -3.0 * fc.invT * fc.M * dm;
        if (f == 0 && dedup) DM[1] = DM[0];
        SP += mult * 3.0 * (sw ? sa : sq);
        SPb += mult * 3.0 * (sw ? sq : sa);
        if (gl == 0) evals += (int64_t)n;
    }
    for (int f = 0; f < 3; ++f) {
        S.DM[f] = group_sum<G>(DM[f], mask);
        S.DMM[f] = S.DMP[f] = S.DMPb[f] = S.Nq[f] = S.Na[f] = 0.0;
    }
    S.SP = group_sum<G>(SP, mask);
    S.SPb = group_sum<G>(SPb, mask);
    S.SL = S.SAN = S.SPP = S.SPPb = S.SPbPb = 0.0;
}

// Float-float pass: the sums of node_pass<..., GRAD, THERMO> (S.DM, S.SP, S.SPb; S.Nq, S.Na,
// S.SAN, S.SL) computed in float-float arithmetic on the FP32 pipe (pnjl_ff.cuh); requires the
// staged float-float tables (nv.p2l != null).  Non-finite sums are returned as such.
template <int G, bool GRAD, bool THERMO, bool HESS = false>
__device__ void node_pass_ff(const NodeView &nv, const PointIn &pt, const double *x, const double *M, int gl,
                             unsigned mask, PassSums &S, int64_t &evals, bool thermo_rt = true) {
    const bool TH = THERMO && thermo_rt;  // THERMO with a run-time switch: one loop serves both
    const bool dedup = (M[1] == M[0]) && (pt.mu[1] == pt.mu[0]);
    const int pn = nv.p_num, n = nv.p_num * nv.t_num;
    const ff xi = ff_from_double(pt.xi);
    const ff z{0.0f, 0.0f};
    ff DM[3] = {z, z, z}, Nq[3] = {z, z, z}, Na[3] = {z, z, z};
    ff DMM[3] = {z, z, z}, DMP[3] = {z, z, z}, DMPb[3] = {z, z, z};
    ff SP = z, SPb = z, SAN = z, SL = z, SPP = z, SPPb = z, SPbPb = z;
#pragma unroll 1
    for (int f = 0; f < 3; ++f) {
        if (f == 1 && dedup) continue;
        bool sw;
        FlavourFF fc = make_flavour_ff(M[f], pt.mu[f], pt.T, x[3], x[4], sw);
        opaque_flavour_ff(fc);
        FlavourAccFF fa;
        fa.zero();
        int ip = gl, it = 0;
        while (ip >= pn) { ip -= pn; ++it; }
        ff sxi = ff_make(1.f), bw = z;
        if (it < nv.t_num) {
            sxi = ff_add_f(ff_mul(xi, ff{nv.c2f[it], nv.c2l[it]}), 1.0f);
            bw = ff{nv.Bf[it], nv.Bl[it]};
        }
#pragma unroll 1
        for (int k = gl; k < n; k += G) {
            const ff q2 = ff_mul(ff{nv.p2f[ip], nv.p2l[ip]}, sxi);
            const ff w = ff_mul(ff{nv.Af[ip], nv.Al[ip]}, bw);
            node_flavour_ff<GRAD, THERMO, HESS>(fc, q2, w, nv.expt, fa, TH);
            ip += G;
            if (ip >= pn) {
                do { ip -= pn; ++it; } while (ip >= pn);
                if (it < nv.t_num) {
                    sxi = ff_add_f(ff_mul(xi, ff{nv.c2f[it], nv.c2l[it]}), 1.0f);
                    bw = ff{nv.Bf[it], nv.Bl[it]};
                }
            }
        }
        const bool two = (f == 0 && dedup);
        auto dbl = [two](ff v) { return two ? ff_mul_f(v, 2.0f) : v; };
        if (GRAD) {
            DM[f] = fa.DM;
            if (two) DM[1] = fa.DM;
            SP = ff_add(SP, dbl(sw ? fa.Sa : fa.Sq));
            SPb = ff_add(SPb, dbl(sw ? fa.Sq : fa.Sa));
        }
        if (HESS) {
            DMM[f] = fa.DMM;
            DMP[f] = sw ? fa.DMa : fa.DMq;
            DMPb[f] = sw ? fa.DMq : fa.DMa;
            if (two) { DMM[1] = DMM[0]; DMP[1] = DMP[0]; DMPb[1] = DMPb[0]; }
            SPP = ff_add(SPP, dbl(sw ? fa.Saa : fa.Sqq));
            SPPb = ff_add(SPPb, dbl(fa.Sqa));
            SPbPb = ff_add(SPbPb, dbl(sw ? fa.Sqq : fa.Saa));
        }
        if (TH) {
            Nq[f] = sw ? fa.Na : fa.Nq;
            Na[f] = sw ? fa.Nq : fa.Na;
            if (two) { Nq[1] = Nq[0]; Na[1] = Na[0]; }
            SAN = ff_add(SAN, dbl(fa.SAN));
            SL = ff_add(SL, dbl(fa.SL));
        }
        if (gl == 0) evals += (int64_t)n;
    }
    for (int f = 0; f < 3; ++f) {
        S.DM[f] = GRAD ? ff_to_double(group_sum_ffv<G>(DM[f], mask)) : 0.0;
        S.Nq[f] = TH ? ff_to_double(group_sum_ffv<G>(Nq[f], mask)) : 0.0;
        S.Na[f] = TH ? ff_to_double(group_sum_ffv<G>(Na[f], mask)) : 0.0;
        S.DMM[f] = HESS ? ff_to_double(group_sum_ffv<G>(DMM[f], mask)) : 0.0;
        S.DMP[f] = HESS ? ff_to_double(group_sum_ffv<G>(DMP[f], mask)) : 0.0;
        S.DMPb[f] = HESS ? ff_to_double(group_sum_ffv<G>(DMPb[f], mask)) : 0.0;
    }
    S.SP = GRAD ? ff_to_double(group_sum_ffv<G>(SP, mask)) : 0.0;
    S.SPb = GRAD ? ff_to_double(group_sum_ffv<G>(SPb, mask)) : 0.0;
    S.SAN = TH ? ff_to_double(group_sum_ffv<G>(SAN, mask)) : 0.0;
    S.SL = TH ? ff_to_double(group_sum_ffv<G>(SL, mask)) : 0.0;
    S.SPP = HESS ? ff_to_double(group_sum_ffv<G>(SPP, mask)) : 0.0;
    S.SPPb = HESS ? ff_to_double(group_sum_ffv<G>(SPPb, mask)) : 0.0;
    S.SPbPb = HESS ? ff_to_double(group_sum_ffv<G>(SPbPb, mask)) : 0.0;
}

// FP64 assembly of Omega, grad, Hessian and thermo from the pass sums and the vacuum terms.
// (An FP32 assembly of the Jacobian for the mixed mode was measured slower: the less
// accurate J32 costs extra FP64 refinement passes.)
// J32: the Hessian block in FP32 arithmetic (the FP32 Newton pass's Jacobian: its sums carry
// ~1e-6 relative error, far above FP32 rounding of the assembly), the gradient in FP64.
template <bool GRAD, bool HESS, bool LOG, bool J32 = false>
__device__ void assemble(const DevParams &P, const PointIn &pt, const double *x, const double *M, const PassSums &S,
                         double V, const double *V1, const double *V2, Eval &ev) {
    const double T = pt.T;
    const double pu = x[0], pd = x[1], ps = x[2], Ph = x[3], Pb = x[4];
    const double G4 = 4.0 * P.G, K2 = 2.0 * P.K, K4 = 4.0 * P.K;
    // chi (Thermodynamics.jl:112-114)
    const double chi = 2.0 * P.G * (pu * pu + pd * pd + ps * ps) - K4 * (pu * pd * ps);
    const double chig[3] = {G4 * pu - K4 * pd * ps, G4 * pd - K4 * pu * ps, G4 * ps - K4 * pu * pd};
    // dM_f/dphi_a
    const double Jm[3][3] = {{-G4, K2 * ps, K2 * pd}, {K2 * ps, -G4, K2 * pu}, {K2 * pd, K2 * pu, -G4}};
    // Polyakov potential U (Thermodynamics.jl:124-130) with safe_log
    const double r = P.T0 / T;
    const double Ta = P.a0 + P.a1 * r + P.a2 * r * r;
    const double Tb = P.b3 * r * r * r;
    const double T4 = (T * T) * (T * T);
    const double pp = Pb * Ph;
    const double g = 1.0 - 6.0 * pp + 4.0 * (Pb * Pb * Pb + Ph * Ph * Ph) - 3.0 * pp * pp;
    const bool gcl = (g <= 0.0) || (g < kPolyakovEps);  // safe_log, Integrals.jl:159-162
    const double lg = gcl ? -36.841361487904734 : log(g);
    const double U = T4 * (-0.5 * Ta * pp + Tb * lg);
    const double gP = -6.0 * Pb + 12.0 * Ph * Ph - 6.0 * Ph * Pb * Pb;
    const double gPb = -6.0 * Ph + 12.0 * Pb * Pb - 6.0 * Ph * Ph * Pb;
    const double ig = gcl ? 0.0 : 1.0 / g;
    const double UP = T4 * (-0.5 * Ta * Pb + Tb * gP * ig);
    const double UPb = T4 * (-0.5 * Ta * Ph + Tb * gPb * ig);
    const double Dsc = -2.0 * T;
    double gO[5];
    for (int a = 0; a < 3; ++a) {
        double s = chig[a];
        for (int f = 0; f < 3; ++f) s += Jm[f][a] * (V1[f] + Dsc * S.DM[f]);
        gO[a] = s;
    }
    gO[3] = UP + Dsc * S.SP;
    gO[4] = UPb + Dsc * S.SPb;
    for (int i = 0; i < 5; ++i) ev.F[i] = -gO[i];
    if (LOG) ev.omega = chi + U + V + Dsc * S.SL;
    else ev.omega = 0.0;
    if (HESS && !J32) {
        double H[5][5];
        const double chih[3][3] = {{G4, -K4 * ps, -K4 * pd}, {-K4 * ps, G4, -K4 * pu}, {-K4 * pd, -K4 * pu, G4}};
        for (int a = 0; a < 3; ++a)
            for (int b = a; b < 3; ++b) {
                double s = chih[a][b];
                for (int f = 0; f < 3; ++f) s += Jm[f][a] * Jm[f][b] * (V2[f] + Dsc * S.DMM[f]);
                H[a][b] = s;
            }
        H[0][1] += (V1[2] + Dsc * S.DM[2]) * K2;
        H[0][2] += (V1[1] + Dsc * S.DM[1]) * K2;
        H[1][2] += (V1[0] + Dsc * S.DM[0]) * K2;
        for (int a = 0; a < 3; ++a) {
            double s3 = 0.0, s4 = 0.0;
            for (int f = 0; f < 3; ++f) {
                s3 += Jm[f][a] * (Dsc * S.DMP[f]);
                s4 += Jm[f][a] * (Dsc * S.DMPb[f]);
            }
            H[a][3] = s3;
            H[a][4] = s4;
        }
        const double gPP = 24.0 * Ph - 6.0 * Pb * Pb;
        const double gPbPb = 24.0 * Pb - 6.0 * Ph * Ph;
        const double gPPb = -6.0 - 12.0 * Ph * Pb;
        const double UPP = gcl ? 0.0 : T4 * Tb * (gPP * ig - gP * gP * ig * ig);
        const double UPbPb = gcl ? 0.0 : T4 * Tb * (gPbPb * ig - gPb * gPb * ig * ig);
        const double UPPb = T4 * (-0.5 * Ta + (gcl ? 0.0 : Tb * (gPPb * ig - gP * gPb * ig * ig)));
        H[3][3] = UPP + Dsc * S.SPP;
        H[3][4] = UPPb + Dsc * S.SPPb;
        H[4][4] = UPbPb + Dsc * S.SPbPb;
        for (int a = 0; a < 5; ++a)
            for (int b = a; b < 5; ++b) {
                ev.J[a * 5 + b] = -H[a][b];
                ev.J[b * 5 + a] = -H[a][b];
            }
    }
    if (HESS && J32) {
        float H[5][5];
        const float g4 = (float)G4, k2 = (float)K2, k4 = (float)K4;
        const float fu = (float)pu, fd = (float)pd, fs = (float)ps, fP = (float)Ph, fPb = (float)Pb;
        const float Jf[3][3] = {{-g4, k2 * fs, k2 * fd}, {k2 * fs, -g4, k2 * fu}, {k2 * fd, k2 * fu, -g4}};
        const float chih[3][3] = {{g4, -k4 * fs, -k4 * fd}, {-k4 * fs, g4, -k4 * fu}, {-k4 * fd, -k4 * fu, g4}};
        const float ds = (float)Dsc;
        float w2[3], w1[3], wp[3], wpb[3];
        for (int f = 0; f < 3; ++f) {
            w2[f] = (float)(V2[f] + Dsc * S.DMM[f]);
            w1[f] = (float)(V1[f] + Dsc * S.DM[f]);
            wp[f] = ds * (float)S.DMP[f];
            wpb[f] = ds * (float)S.DMPb[f];
        }
        for (int a = 0; a < 3; ++a)
            for (int b = a; b < 3; ++b) {
                float sab = chih[a][b];
                for (int f = 0; f < 3; ++f) sab += Jf[f][a] * Jf[f][b] * w2[f];
                H[a][b] = sab;
            }
        H[0][1] += w1[2] * k2;
        H[0][2] += w1[1] * k2;
        H[1][2] += w1[0] * k2;
        for (int a = 0; a < 3; ++a) {
            float s3 = 0.0f, s4 = 0.0f;
            for (int f = 0; f < 3; ++f) {
                s3 += Jf[f][a] * wp[f];
                s4 += Jf[f][a] * wpb[f];
            }
            H[a][3] = s3;
            H[a][4] = s4;
        }
        const float t4 = (float)T4, tb = (float)Tb, ta = (float)Ta, igf = (float)ig;
        const float gPf = (float)gP, gPbf = (float)gPb;
        const float gPP = 24.0f * fP - 6.0f * fPb * fPb;
        const float gPbPb = 24.0f * fPb - 6.0f * fP * fP;
        const float gPPb = -6.0f - 12.0f * fP * fPb;
        const float UPP = gcl ? 0.0f : t4 * tb * (gPP * igf - gPf * gPf * igf * igf);
        const float UPbPb = gcl ? 0.0f : t4 * tb * (gPbPb * igf - gPbf * gPbf * igf * igf);
        const float UPPb = t4 * (-0.5f * ta + (gcl ? 0.0f : tb * (gPPb * igf - gPf * gPbf * igf * igf)));
        H[3][3] = UPP + ds * (float)S.SPP;
        H[3][4] = UPPb + ds * (float)S.SPPb;
        H[4][4] = UPbPb + ds * (float)S.SPbPb;
        for (int a = 0; a < 5; ++a)
            for (int b = a; b < 5; ++b) {
                ev.J[a * 5 + b] = -(double)H[a][b];
                ev.J[b * 5 + a] = -(double)H[a][b];
            }
    }
    if (LOG) {
        // dU/dT (Thermodynamics.jl:142-163) and dD/dT = -2 sum wL + 6 sum w (a n+ + b n-)
        const double dTa = -P.a1 * P.T0 / (T * T) - 2.0 * P.a2 * P.T0 * P.T0 / (T * T * T);
        const double dTb = -3.0 * P.b3 * P.T0 * P.T0 * P.T0 / (T4);
        const double UT = 4.0 * T * T * T * (-0.5 * Ta * pp + Tb * lg) + T4 * (dTa * (-0.5 * pp) + dTb * lg);
        ev.dOdT = UT - 2.0 * S.SL + 6.0 * S.SAN;
        for (int f = 0; f < 3; ++f) {
            ev.rho[f] = 6.0 * (S.Nq[f] - S.Na[f]);
            ev.nq[f] = 2.0 * P.Nc * S.Nq[f];
            ev.naq[f] = 2.0 * P.Nc * S.Na[f];
        }
    }
}

// ---------------------------------------------------------------------------------------
// 5x5 dense LU with partial pivoting (first maximal pivot, as LAPACK getrf); returns
// false when a pivot is exactly zero (Julia's SingularException).  FAST (the mixed solver's
// FP32-phase steps): each pivot's reciprocal is taken once, by rcp_normal, and multiplied in
// -- LAPACK's dgetf2 scales the column by the pivot's reciprocal the same way -- instead of
// 15 IEEE divisions.
// |v| as a bit pattern: orders like the value for non-negative doubles; NaN above +inf.
__device__ __forceinline__ unsigned long long abs_bits(double v) {
    return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}

// Whether the root with Jacobian J = Hessian_x P (= -Hessian_x Omega, 5 x 5) lies on an
// unstable branch: det J < 0.  A thermodynamically stable root -- the min-Omega phase, or a
// metastable one -- has exactly one negative eigenvalue of Hessian_x Omega, the saddle of the
// Polyakov-loop potential in (Phi, Phibar), so det J > 0; the branch between two coexisting
// phases has a second one.  (Checked with the oracle's Hessians on 600 random points of the
// (T, mu, xi) boxes of the scans: every min-Omega root has one negative eigenvalue, every
// root with two has det J < 0.)  Elimination with partial pivoting on a copy; a singular or
// non-finite J counts as unstable.
static __device__ __noinline__ bool det5_negative(const double *Jin) {
    double A[25];
#pragma unroll
    for (int i = 0; i < 25; ++i) A[i] = Jin[i];
    bool neg = false;
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        int p = c;
        double big = fabs(A[c * 5 + c]);
#pragma unroll
        for (int r = c + 1; r < 5; ++r) {
            const double v = fabs(A[r * 5 + c]);
            if (v > big) { big = v; p = r; }
        }
        if (!(big > 0.0 && big <= 1.7976931348623157e308)) return true;
#pragma unroll
        for (int r = c + 1; r < 5; ++r)
            if (r == p) {
#pragma unroll
                for (int k = c; k < 5; ++k) {
                    const double t = A[c * 5 + k];
                    A[c * 5 + k] = A[r * 5 + k];
                    A[r * 5 + k] = t;
                }
                neg = !neg;
            }
        const double d = A[c * 5 + c];
        if (d < 0.0) neg = !neg;
        const double inv = 1.0 / d;
#pragma unroll
        for (int r = c + 1; r < 5; ++r) {
            const double f = A[r * 5 + c] * inv;
#pragma unroll
            for (int k = c + 1; k < 5; ++k) A[r * 5 + k] = fma(-f, A[c * 5 + k], A[r * 5 + k]);
        }
    }
    return neg;
}

template <bool FAST = false>
__device__ __forceinline__ bool lu_solve5(const double *Ain, const double *b, double *x) {
    double A[25], y[5], inv[5];
#pragma unroll
    for (int i = 0; i < 25; ++i) A[i] = Ain[i];
#pragma unroll
    for (int i = 0; i < 5; ++i) y[i] = b[i];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        int p = k;
        if (FAST) {  // the same first maximal pivot, compared on the bit patterns (integer pipe)
            unsigned long long bb = abs_bits(A[k * 5 + k]);
#pragma unroll
            for (int i = k + 1; i < 5; ++i) {
                const unsigned long long v = abs_bits(A[i * 5 + k]);
                if (v > bb) { bb = v; p = i; }
            }
            if (bb == 0) return false;
        } else {
            double best = fabs(A[k * 5 + k]);
#pragma unroll
            for (int i = k + 1; i < 5; ++i) {
                const double v = fabs(A[i * 5 + k]);
                if (v > best) { best = v; p = i; }
            }
            if (A[p * 5 + k] == 0.0) return false;
        }
        if (p != k) {
#pragma unroll
            for (int j = 0; j < 5; ++j) {
                const double t = A[k * 5 + j];
                A[k * 5 + j] = A[p * 5 + j];
                A[p * 5 + j] = t;
            }
            const double t = y[k];
            y[k] = y[p];
            y[p] = t;
        }
        if (FAST) inv[k] = rcp_normal(A[k * 5 + k]);
#pragma unroll
        for (int i = k + 1; i < 5; ++i) {
            const double l = FAST ? A[i * 5 + k] * inv[k] : A[i * 5 + k] / A[k * 5 + k];
            A[i * 5 + k] = l;
#pragma unroll
            for (int j = k + 1; j < 5; ++j) A[i * 5 + j] -= l * A[k * 5 + j];
            y[i] -= l * y[k];
        }
    }
#pragma unroll
    for (int i = 4; i >= 0; --i) {
        double s = y[i];
#pragma unroll
        for (int j = i + 1; j < 5; ++j) s -= A[i * 5 + j] * y[j];
        y[i] = FAST ? s * inv[i] : s / A[i * 5 + i];
    }
#pragma unroll
    for (int i = 0; i < 5; ++i) x[i] = y[i];
    return true;
}

// LU factorization with partial pivoting kept for repeated solves (mixed-precision
// refinement reuses one FP32-assembled Jacobian); false when a pivot is exactly zero.
__device__ __forceinline__ bool lu_factor5(const double *Ain, double *A, int *piv) {
#pragma unroll
    for (int i = 0; i < 25; ++i) A[i] = Ain[i];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        int p = k;
        double best = fabs(A[k * 5 + k]);
#pragma unroll
        for (int i = k + 1; i < 5; ++i) {
            const double v = fabs(A[i * 5 + k]);
            if (v > best) { best = v; p = i; }
        }
        piv[k] = p;
        if (A[p * 5 + k] == 0.0) return false;
        if (p != k) {
#pragma unroll
            for (int j = 0; j < 5; ++j) {
                const double t = A[k * 5 + j];
                A[k * 5 + j] = A[p * 5 + j];
                A[p * 5 + j] = t;
            }
        }
        const double inv = 1.0 / A[k * 5 + k];
#pragma unroll
        for (int i = k + 1; i < 5; ++i) {
            const double l = A[i * 5 + k] * inv;
            A[i * 5 + k] = l;
#pragma unroll
            for (int j = k + 1; j < 5; ++j) A[i * 5 + j] -= l * A[k * 5 + j];
        }
    }
    return true;
}

__device__ __forceinline__ void lu_solve_factored5(const double *A, const int *piv, const double *b, double *x) {
    double y[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) y[i] = b[i];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        const int p = piv[k];
        if (p != k) { const double t = y[k]; y[k] = y[p]; y[p] = t; }
#pragma unroll
        for (int i = k + 1; i < 5; ++i) y[i] -= A[i * 5 + k] * y[k];
    }
#pragma unroll
    for (int i = 4; i >= 0; --i) {
        double s = y[i];
#pragma unroll
        for (int j = i + 1; j < 5; ++j) s -= A[i * 5 + j] * y[j];
        y[i] = s / A[i * 5 + i];
    }
#pragma unroll
    for (int i = 0; i < 5; ++i) x[i] = y[i];
}

// The 5-vector checks on the bit patterns (integer pipe; the FP64 pipe is the scarce one):
// |v| as the pattern without the sign orders like the value for non-negative doubles, and a
// NaN's pattern is above +inf's.
__device__ __forceinline__ double norm_inf5(const double *v) {
    unsigned long long m = 0;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        const unsigned long long b = abs_bits(v[i]);
        m = b > m ? b : m;
    }
    // NaN if any component is NaN (its pattern is the largest)
    return m > 0x7ff0000000000000ull ? __longlong_as_double(0x7ff8000000000000ll) : __longlong_as_double((long long)m);
}
__device__ __forceinline__ bool any_nan5(const double *v) {
    bool r = false;
#pragma unroll
    for (int i = 0; i < 5; ++i) r |= abs_bits(v[i]) > 0x7ff0000000000000ull;
    return r;
}
__device__ __forceinline__ bool all_finite5(const double *v) {
    bool r = true;
#pragma unroll
    for (int i = 0; i < 5; ++i) r &= abs_bits(v[i]) < 0x7ff0000000000000ull;
    return r;
}

// Outcome of one NLsolve run plus the postprocessed candidate at its final x.
struct Candidate {
    double x[5];
    double residual_norm;
    int iterations;
    bool f_converged, exception, phys;
    bool unstable = false;  // the root lies on an unstable branch (det5_negative)
    double omega, entropy, rho[3], nq[3], naq[3];
};

__device__ __forceinline__ void postprocess(const DevParams &P, const PointIn &pt, const SolveOpts &o, const Eval &ev,
                                            Candidate &c) {
    double M[3];
    masses(P, c.x, M);
    c.omega = ev.omega;
    c.entropy = -ev.dOdT;
    for (int f = 0; f < 3; ++f) { c.rho[f] = ev.rho[f]; c.nq[f] = ev.nq[f]; c.naq[f] = ev.naq[f]; }
    const double pressure = -ev.omega;
    const double rho_norm = (c.rho[0] + c.rho[1] + c.rho[2]) / (3.0 * P.rho0);
    const double energy = -pressure + (pt.mu[0] * c.rho[0] + pt.mu[1] * c.rho[1] + pt.mu[2] * c.rho[2]) + pt.T * c.entropy;
    const double Ph = c.x[3], Pb = c.x[4], tol = o.phi_tol;
    bool ok = isfinite(Ph) && isfinite(Pb) && (-tol <= Ph) && (Ph <= 1.0 + tol) && (-tol <= Pb) && (Pb <= 1.0 + tol);
    for (int f = 0; f < 3; ++f) ok = ok && isfinite(M[f]) && (M[f] > 0.0);
    ok = ok && isfinite(c.omega) && isfinite(pressure) && isfinite(rho_norm) && isfinite(c.entropy) && isfinite(energy);
    c.phys = ok;
}

__device__ __forceinline__ bool cand_good(const Candidate &c, double rmax) {
    return c.f_converged && isfinite(c.residual_norm) && c.residual_norm <= rmax && c.phys;
}

// _choose_candidate (ImplicitSolver.jl:72-101): true -> take the fallback
__device__ __forceinline__ bool choose_fallback(const Candidate &p, const Candidate &f, double rmax) {
    const bool pg = cand_good(p, rmax), fg = cand_good(f, rmax);
    if (fg && !pg) return true;
    if (pg && !fg) return false;
    if (fg && pg) {
        if (f.omega < p.omega) return true;
        if (f.omega > p.omega) return false;
        return f.residual_norm < p.residual_norm;
    }
    if (f.f_converged && !p.f_converged) return true;
    if (p.f_converged && !f.f_converged) return false;
    if (isfinite(f.residual_norm) && isfinite(p.residual_norm)) return f.residual_norm < p.residual_norm;
    return false;
}

}  // namespace pnjl
