// pnjl_ff.cuh -- float-float ("double-single") residual pass of the mixed-precision solver.
//
// A float-float number is an unevaluated sum hi + lo of two FP32 values (|lo| <= ulp(hi)/2),
// about 44-48 significant bits.  Its arithmetic runs on the FP32 pipe, which on this GPU has
// 64x the FP64 rate, so one float-float pass over the nodes costs a small fraction of an FP64
// pass.  The mixed solver uses it for exactly one thing: the residual F(x32) at the FP32 root,
// accurate to ~1e-12, from which one FP64-Jacobian-free correction step lands within the FP64
// certification radius.  Convergence is still certified by an FP64 residual pass (and the
// thermodynamics come from that FP64 pass), so this pass only saves the FP64 residual pass
// that used to precede the correction step.
//
// Error-free transformations (Knuth's TwoSum, Dekker's Fast2Sum, the FMA product), the
// float-float add and multiply follow the published double-single / double-double algorithms
// (Dekker 1971; Hida, Li and Bailey, "Library for double-double and quad-double arithmetic",
// 2007).  exp is table-driven in the manner of Tang (ACM TOMS 15, 1989): e^x = e^n e^(j/16) e^g
// with n integer, |g| <= 1/32 and a degree-7 Taylor polynomial.  Reciprocal and reciprocal
// square root are one Newton step from the correctly rounded FP32 value.
#pragma once

#include <cuda_runtime.h>

#include "pnjl_f64.cuh"

namespace pnjl {

struct ff {
    float h, l;
};

// Function tables in shared memory, as (h, l) float pairs: e^k (k = -kExpMaxN..kExpMaxN),
// e^(j/256) (j = 0..255), ln c_j and 1/c_j for c_j = 1 + (2j + 1)/256 (j = 0..127); then (from
// float kExp64Offset, 8-byte aligned) the kExp64N doubles 2^(j/256) of the FP64 exponential
// (pnjl_f64.cuh).
constexpr int kExpMaxN = 88;
constexpr int kExpIntN = 2 * kExpMaxN + 1;
constexpr int kExpFracN = 256;
constexpr int kLogN = 128;
constexpr int kExpFracOff = 2 * kExpIntN;             // floats
constexpr int kLogOff = kExpFracOff + 2 * kExpFracN;  // ln c_j pairs, then 1/c_j pairs
constexpr int kExp64Offset = kLogOff + 4 * kLogN;
constexpr int kExpTableFloats = kExp64Offset + 2 * kExp64N;
static_assert(kExp64Offset % 2 == 0, "FP64 table alignment");

__device__ __forceinline__ ff ff_make(float h) { return ff{h, 0.0f}; }
__device__ __forceinline__ ff ff_from_float_pair(float h, float l) { return ff{h, l}; }
__device__ __forceinline__ ff ff_from_double(double d) {
    const float h = __double2float_rn(d);
    return ff{h, __double2float_rn(d - (double)h)};
}
__device__ __forceinline__ double ff_to_double(ff a) { return (double)a.h + (double)a.l; }

__device__ __forceinline__ ff two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return ff{s, e};
}
__device__ __forceinline__ ff fast_two_sum(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return ff{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return ff{p, __fmaf_rn(a, b, -p)};
}
// a + b with relative error ~2^-47 of the result (two TwoSums; 20 FP32 additions): for the
// lane reductions of the pass sums
__device__ __forceinline__ ff ff_add_acc(ff a, ff b) {
    const ff s = two_sum(a.h, b.h);
    const ff t = two_sum(a.l, b.l);
    ff r = fast_two_sum(s.h, __fadd_rn(s.l, t.h));
    return fast_two_sum(r.h, __fadd_rn(r.l, t.l));
}
// a + b with absolute error ~2^-47 (|a| + |b|) (one TwoSum on the high parts; 11 FP32
// additions).  In the node integrand every operand already carries a relative error of that
// size from its own float-float rounding, so the cheaper form loses nothing there: where a
// and b cancel, their own errors dominate either way.
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    const ff s = two_sum(a.h, b.h);
    return fast_two_sum(s.h, __fadd_rn(__fadd_rn(s.l, a.l), b.l));
}
__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.h, -a.l}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }
__device__ __forceinline__ ff ff_add_f(ff a, float b) {
    const ff s = two_sum(a.h, b);
    return fast_two_sum(s.h, __fadd_rn(s.l, a.l));
}
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const ff p = two_prod(a.h, b.h);
    float e = __fmaf_rn(a.h, b.l, p.l);
    e = __fmaf_rn(a.l, b.h, e);
    return fast_two_sum(p.h, e);
}
__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
    const ff p = two_prod(a.h, b);
    return fast_two_sum(p.h, __fmaf_rn(a.l, b, p.l));
}
__device__ __forceinline__ ff ff_sel(bool c, ff a, ff b) { return ff{c ? a.h : b.h, c ? a.l : b.l}; }

// 1/b: one Newton step y = y0 + y0 e, e = 1 - b y0, from the hardware FP32 reciprocal y0
// (~1 ulp).  1 - b.h y0 is exactly representable (|e| < 2^-22 with bits down to 2^-47), so
// one FMA gives it; the b.l term is small.  Relative error ~e^2 + 2^-48.
__device__ __forceinline__ ff ff_rcp(ff b) {
    float y0;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y0) : "f"(b.h));
    float e = __fmaf_rn(-b.h, y0, 1.0f);
    e = __fmaf_rn(-b.l, y0, e);
    return fast_two_sum(y0, __fmul_rn(y0, e));
}

// 1/sqrt(x): y = y0 (1 + e/2 + 3e^2/8), e = 1 - x y0^2, from the hardware FP32 value y0
// (~2 ulp; y0^2 exact as a pair, 1 - x.h y0^2 within 2^-47 in one FMA; the remainder of the
// series is ~e^3).
__device__ __forceinline__ ff ff_rsqrt(ff x) {
    const float y0 = rsqrtf(x.h);
    const ff p = two_prod(y0, y0);
    float e = __fmaf_rn(-x.h, p.h, 1.0f);
    e = __fmaf_rn(-x.h, p.l, e);
    e = __fmaf_rn(-x.l, p.h, e);
    return fast_two_sum(y0, __fmul_rn(__fmul_rn(y0, e), __fmaf_rn(e, 0.375f, 0.5f)));
}

// e^x for |x| <= 88 (0 below, +inf above), a table method: x = n + j/256 + g with
// n + j/256 = round(256 x)/256 (j = 0..255) and |g| <= 1/512; e^x = e^n e^(j/256) e^g with
// e^g = 1 + g + g^2/2 + g^3 (1/6 + g/24) -- the remainder g^5/120 is below 2.5e-16 -- where
// g^2/2 is kept exact as a pair and the cubic tail, below 1.3e-9, in FP32.
__device__ __forceinline__ ff ff_exp(ff x, const float *tab) {
    if (!(x.h > -88.0f)) return ff{0.0f, 0.0f};
    if (!(x.h < 88.0f)) return ff{__int_as_float(0x7f800000), 0.0f};
    const float mf = rintf(x.h * 256.0f);
    const int m = (int)mf;
    const int n = m >> 8, j = m & 255;                    // m = 256 n + j
    const ff g = two_sum(__fsub_rn(x.h, mf * 0.00390625f), x.l);  // x.h - m/256 is exact
    ff q = two_prod(g.h, g.h);                            // g^2 (+ the g.h g.l cross term)
    q.l = __fmaf_rn(2.0f * g.h, g.l, q.l);
    const float tail = __fmul_rn(__fmul_rn(q.h, g.h), __fmaf_rn(g.h, 1.0f / 24.0f, 1.0f / 6.0f));
    const ff s = two_sum(1.0f, g.h);
    const ff eg = ff_add(s, ff{0.5f * q.h, __fadd_rn(__fadd_rn(0.5f * q.l, g.l), tail)});
    const ff en{tab[2 * (n + kExpMaxN)], tab[2 * (n + kExpMaxN) + 1]};
    const ff ej{tab[kExpFracOff + 2 * j], tab[kExpFracOff + 2 * j + 1]};
    return ff_mul(ff_mul(en, ej), eg);
}

// ln x for positive normal x: x = 2^k m (m in [1, 2)), c the centre of m's 1/128-wide
// interval, u = (m - c)/c with |u| <= 1/257, ln x = k ln2 + ln c + log1p(u),
// log1p(u) = u - u^2/2 + u^3 (1/3 - u/4 + u^2/5 - u^3/6) (remainder below 3e-17), with u^2
// exact as a pair and the cubic tail in FP32.
__device__ __forceinline__ ff ff_log(ff x, const float *tab) {
    if (!(x.h >= 1.17549435e-38f && x.h < 1.7014118e38f)) return ff{__int_as_float(0x7fc00000), 0.0f};
    const unsigned b = __float_as_uint(x.h);
    const int k = (int)((b >> 23) & 0xffu) - 127;
    const int j = (int)((b >> 16) & 0x7fu);               // top 7 bits of the significand
    const float mh = __uint_as_float((b & 0x007fffffu) | 0x3f800000u);
    const float ml = __fmul_rn(x.l, __uint_as_float((unsigned)(127 - k) << 23));  // x.l 2^-k (exact)
    const float c = __fmaf_rn((float)j, 0.0078125f, 1.00390625f);                 // 1 + (2j + 1)/256
    const ff d = two_sum(__fsub_rn(mh, c), ml);           // m - c (the subtraction is exact)
    const ff u = ff_mul(d, ff{tab[kLogOff + 2 * kLogN + 2 * j], tab[kLogOff + 2 * kLogN + 2 * j + 1]});
    ff q = two_prod(u.h, u.h);
    q.l = __fmaf_rn(2.0f * u.h, u.l, q.l);
    const float p = __fmaf_rn(__fmaf_rn(__fmaf_rn(u.h, -1.0f / 6.0f, 0.2f), u.h, -0.25f), u.h, 1.0f / 3.0f);
    const float tail = __fmul_rn(__fmul_rn(q.h, u.h), p);
    const ff l1p = ff_add(u, ff{-0.5f * q.h, __fadd_rn(-0.5f * q.l, tail)});
    const ff kl = ff_mul_f(ff{0x1.62e43p-1f, -0x1.05c61p-29f}, (float)k);  // k ln2 (ln2 as a pair)
    const ff lc{tab[kLogOff + 2 * j], tab[kLogOff + 2 * j + 1]};
    return ff_add(ff_add(kl, lc), l1p);
}

// Per-flavour constants of a float-float pass (the same branch-free form as FlavourConst).
struct FlavourFF {
    ff M, M2, mu, invT, C, C2;
    ff Pq, Pa, Pq2, Pa2;
    ff k1_0, k2_0, k1_1, k2_1;
    ff e3_0, e2_0, e1_0, e2_1, e1_1, e0_1;
};

__device__ __forceinline__ FlavourFF make_flavour_ff(double M, double mu, double T, double Phi, double Phib,
                                                     bool &swapped) {
    FlavourFF fc;
    swapped = mu < 0.0;
    const double mua = swapped ? -mu : mu;
    const double Pq = swapped ? Phib : Phi;
    const double Pa = swapped ? Phi : Phib;
    const double C = exp(-2.0 * mua / T);
    fc.M = ff_from_double(M);
    fc.M2 = ff_from_double(M * M);
    fc.mu = ff_from_double(mua);
    fc.invT = ff_from_double(1.0 / T);
    fc.C = ff_from_double(C);
    fc.C2 = ff_from_double(C * C);
    fc.Pq = ff_from_double(Pq);
    fc.Pa = ff_from_double(Pa);
    fc.Pq2 = ff_from_double(2.0 * Pq);
    fc.Pa2 = ff_from_double(2.0 * Pa);
    fc.k1_0 = ff_from_double(3.0 * Pq);
    fc.k2_0 = ff_from_double(3.0 * Pa);
    fc.k1_1 = fc.k2_0;
    fc.k2_1 = fc.k1_0;
    fc.e3_0 = ff_from_double(C * C * C);
    fc.e2_0 = ff_from_double(3.0 * Pq * C * C);
    fc.e1_0 = ff_from_double(3.0 * Pa * C);
    fc.e2_1 = fc.e1_0;
    fc.e1_1 = fc.e2_0;
    fc.e0_1 = fc.e3_0;
    return fc;
}

__device__ __forceinline__ void opaque(ff &v) { asm volatile("" : "+f"(v.h), "+f"(v.l)); }
// the per-flavour constants as opaque register values for the node loop (see opaque())
__device__ __forceinline__ void opaque_flavour_ff(FlavourFF &fc) {
    opaque(fc.M); opaque(fc.M2); opaque(fc.mu); opaque(fc.invT); opaque(fc.C); opaque(fc.C2);
    opaque(fc.Pq); opaque(fc.Pa); opaque(fc.Pq2); opaque(fc.Pa2);
    opaque(fc.k1_0); opaque(fc.k2_0); opaque(fc.k1_1); opaque(fc.k2_1);
    opaque(fc.e3_0); opaque(fc.e2_0); opaque(fc.e1_0); opaque(fc.e2_1); opaque(fc.e1_1); opaque(fc.e0_1);
}

// Per-flavour sums of a float-float pass: gradient terms dD/dM, dD/dPhi, dD/dPhibar (quark /
// antiquark side) and thermo terms (number sums, a n+ + b n-, log term).
struct FlavourAccFF {
    ff DM, Sq, Sa, Nq, Na, SAN, SL;
    ff DMM, DMq, DMa, Sqq, Sqa, Saa;  // second derivatives (Newton passes)
    __device__ __forceinline__ void zero() {
        DM = Sq = Sa = Nq = Na = SAN = SL = ff{0.0f, 0.0f};
        DMM = DMq = DMa = Sqq = Sqa = Saa = ff{0.0f, 0.0f};
    }
};

// One node-flavour evaluation (node_flavour<..., GRAD, HESS, THERMO> of pnjl_device.cuh in
// float-float), with the reference's clamps max(f, 1e-16) decided on the leading parts.
template <bool GRAD, bool THERMO, bool HESS = false>
__device__ __forceinline__ void node_flavour_ff(const FlavourFF &fc, ff q2, ff w, const float *etab,
                                                FlavourAccFF &acc, bool thermo = true) {
    const ff E2 = ff_add(q2, fc.M2);
    const ff rE = ff_rsqrt(E2);
    const ff E = ff_mul(E2, rE);
    const ff a = ff_mul(ff_sub(fc.mu, E), fc.invT);
    const bool sig = a.h > 0.0f;
    const ff t = ff_exp(sig ? ff_neg(a) : a, etab);
    const ff t2 = ff_mul(t, t);
    const ff t3 = ff_mul(t2, t);
    const ff k1 = ff_sel(sig, fc.k1_1, fc.k1_0);
    const ff k2 = ff_sel(sig, fc.k2_1, fc.k2_0);
    const ff fp = ff_add_f(ff_mul(ff_add(ff_mul(ff_add(t, k2), t), k1), t), 1.0f);
    const ff e3 = ff_sel(sig, ff_make(1.0f), fc.e3_0);
    const ff e2 = ff_sel(sig, fc.e2_1, fc.e2_0);
    const ff e1 = ff_sel(sig, fc.e1_1, fc.e1_0);
    const ff e0 = ff_sel(sig, fc.e0_1, ff_make(1.0f));
    const ff gm = ff_add(ff_mul(ff_add(ff_mul(ff_add(ff_mul(e3, t), e2), t), e1), t), e0);
    const float alpha3 = sig ? t3.h : 1.0f;
    const bool clP = fp.h < 1e-16f;
    const bool clM = gm.h < 1e-16f * alpha3;
    const ff fpc = clP ? ff_make(1.0f) : fp;
    const ff gmc = clM ? ff_make(1.0f) : gm;
    const ff ip = clP ? ff_make(0.0f) : ff_rcp(fpc);
    const ff im = clM ? ff_make(0.0f) : ff_rcp(gmc);
    const ff u1 = ff_sel(sig, t2, t);
    const ff u2 = ff_sel(sig, t, t2);
    const ff u3 = ff_sel(sig, ff_make(1.0f), t3);
    const ff r1 = ff_mul(u1, ip), r2 = ff_mul(u2, ip), r3 = ff_mul(u3, ip);
    const ff Cim = ff_mul(fc.C, im);
    const ff s1 = ff_mul(u1, Cim);
    const ff s2 = ff_mul(fc.C, ff_mul(u2, Cim));
    const ff s3 = ff_mul(fc.C2, ff_mul(u3, Cim));
    const ff np = clP ? ff_make(sig ? 1.0f : 0.0f) : ff_add(ff_add(ff_mul(fc.Pq, r1), ff_mul(fc.Pa2, r2)), r3);
    const ff nm = clM ? ff_make(0.0f) : ff_add(ff_add(ff_mul(fc.Pa, s1), ff_mul(fc.Pq2, s2)), s3);
    if (GRAD || HESS) {
        const ff mE = ff_mul(fc.M, rE);
        const ff LE = ff_mul_f(ff_mul(ff_add(np, nm), fc.invT), -3.0f);
        if (GRAD) {
            acc.DM = ff_add(acc.DM, ff_mul(w, ff_mul(LE, mE)));
            acc.Sq = ff_add(acc.Sq, ff_mul_f(ff_mul(w, ff_add(r1, s2)), 3.0f));
            acc.Sa = ff_add(acc.Sa, ff_mul_f(ff_mul(w, ff_add(r2, s1)), 3.0f));
        }
        if (HESS) {
            const ff one = ff_make(1.0f);
            const ff Laa = clP ? ff_make(0.0f)
                               : ff_sub(ff_add(ff_add(ff_mul_f(ff_mul(fc.Pq, r1), 3.0f), ff_mul_f(ff_mul(fc.Pa, r2), 12.0f)),
                                               ff_mul_f(r3, 9.0f)),
                                        ff_mul_f(ff_mul(np, np), 9.0f));
            const ff Lbb = clM ? ff_make(0.0f)
                               : ff_sub(ff_add(ff_add(ff_mul_f(ff_mul(fc.Pa, s1), 3.0f), ff_mul_f(ff_mul(fc.Pq, s2), 12.0f)),
                                               ff_mul_f(s3, 9.0f)),
                                        ff_mul_f(ff_mul(nm, nm), 9.0f));
            const ff iT2 = ff_mul(fc.invT, fc.invT);
            const ff LEE = ff_mul(ff_add(Laa, Lbb), iT2);
            const ff mE2 = ff_mul(mE, mE);
            const ff LMM = ff_add(ff_mul(LEE, mE2), ff_mul(ff_mul(LE, ff_sub(one, mE2)), rE));
            const ff np3 = ff_mul_f(np, 3.0f), nm3 = ff_mul_f(nm, 3.0f);
            const ff LEq = ff_neg(ff_mul(fc.invT, ff_mul_f(ff_add(ff_mul(r1, ff_sub(one, np3)),
                                                                 ff_mul(s2, ff_sub(ff_make(2.0f), nm3))), 3.0f)));
            const ff LEa = ff_neg(ff_mul(fc.invT, ff_mul_f(ff_add(ff_mul(r2, ff_sub(ff_make(2.0f), np3)),
                                                                 ff_mul(s1, ff_sub(one, nm3))), 3.0f)));
            acc.DMM = ff_add(acc.DMM, ff_mul(w, LMM));
            acc.DMq = ff_add(acc.DMq, ff_mul(w, ff_mul(LEq, mE)));
            acc.DMa = ff_add(acc.DMa, ff_mul(w, ff_mul(LEa, mE)));
            acc.Sqq = ff_add(acc.Sqq, ff_mul_f(ff_mul(w, ff_add(ff_mul(r1, r1), ff_mul(s2, s2))), -9.0f));
            acc.Sqa = ff_add(acc.Sqa, ff_mul_f(ff_mul(w, ff_add(ff_mul(r1, r2), ff_mul(s1, s2))), -9.0f));
            acc.Saa = ff_add(acc.Saa, ff_mul_f(ff_mul(w, ff_add(ff_mul(r2, r2), ff_mul(s1, s1))), -9.0f));
        }
    }
    if (THERMO && thermo) {
        acc.Nq = ff_add(acc.Nq, ff_mul(w, np));
        acc.Na = ff_add(acc.Na, ff_mul(w, nm));
        const ff b = ff_sub(a, ff_mul_f(ff_mul(fc.mu, fc.invT), 2.0f));
        acc.SAN = ff_add(acc.SAN, ff_mul(w, ff_add(ff_mul(a, np), ff_mul(b, nm))));
        // ln f+ + ln f- = 6 max(a,0) + ln(fp gm); a clamped factor is replaced by the
        // reference's constant (log(1e-16), plus 3a in its rescaled quark branch)
        ff L = ff_log(ff_mul(fpc, gmc), etab);
        if (sig) L = ff_add(L, ff_mul_f(a, 6.0f));
        if (clP) L = ff_add(L, ff_from_float_pair(-36.84136199951171875f, 5.11606970e-07f));
        if (clM) {
            L = ff_add(L, ff_from_float_pair(-36.84136199951171875f, 5.11606970e-07f));
            if (sig) L = ff_sub(L, ff_mul_f(a, 3.0f));
        }
        acc.SL = ff_add(acc.SL, ff_mul(w, L));
    }
}

// Butterfly sum of a float-float value over the lanes of a group (every lane ends with the
// same bits: a + b and b + a are computed by the same operation order on both partners only
// up to commutativity of TwoSum, which is exact, so the results are identical).
template <int G>
__device__ __forceinline__ ff group_sum_ffv(ff v, unsigned mask) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        const ff u{__shfl_xor_sync(mask, v.h, o), __shfl_xor_sync(mask, v.l, o)};
        v = ff_add_acc(v, u);
    }
    return v;
}

}  // namespace pnjl
