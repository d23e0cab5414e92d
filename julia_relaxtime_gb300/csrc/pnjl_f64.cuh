// pnjl_f64.cuh -- FP64 exponential, reciprocal and reciprocal square root for the FP64
// residual (certification) pass of the mixed-precision solve.
//
// On the GB300 the FP64 pipe is the scarcest unit (about 2 FP64 FMA per clock per SM): every
// FP64 instruction of that pass costs 64 issue cycles of an SM sub-partition.  These
// functions take fewer FP64 instructions than the general-purpose library calls on the
// arguments the pass meets, within about 1 ulp; every other argument (non-finite, extreme
// exponents) is handed to the library function in a call kept out of line.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace pnjl {

// 2^(j/256), j = 0..255, rounded to double (host-built table, staged in shared memory)
constexpr int kExp64Bits = 8;
constexpr int kExp64N = 1 << kExp64Bits;

// Cody-Waite split of ln2/256: kLn2HiD = (ln2 truncated to 33 significant bits)/256, so that
// k * kLn2HiD is exact for |k| < 2^20; kLn2LoD = the rest of ln2/256, rounded.
constexpr double kInvLn2xN = 0x1.71547652b82fep+8;  // 256/ln2
constexpr double kLn2HiD = 0x1.62e42fefp-9;
constexpr double kLn2LoD = 0x1.473de6af278edp-42;
constexpr double kRoundShifter = 0x1.8p52;           // 1.5*2^52: adding it rounds to an integer

// c ? a : b as a 64-bit integer select (selp.b64).  The compiler otherwise turns some
// selects between FP64 values into FP64 arithmetic; measured in the certification pass.
__device__ __forceinline__ double dsel(bool c, double a, double b) {
    long long r;
    asm("{\n\t.reg .pred p;\n\tsetp.ne.s32 p, %3, 0;\n\tselp.b64 %0, %1, %2, p;\n\t}"
        : "=l"(r)
        : "l"(__double_as_longlong(a)), "l"(__double_as_longlong(b)), "r"((int)c));
    return __longlong_as_double(r);
}

// Marks a loop invariant as an opaque register value.  Without it the compiler recomputes
// products of invariants (3 Phi, 2 Phi C, ...) inside the node loop to save registers, which
// in the certification pass cost about 15 extra FP64 instructions per node-flavour (measured:
// 72 -> 57 per node-flavour, 26 % less time).
__device__ __forceinline__ void opaque(double &v) { asm volatile("" : "+d"(v)); }
__device__ __forceinline__ void opaque(float &v) { asm volatile("" : "+f"(v)); }

static __device__ __noinline__ double exp_library(double x) { return exp(x); }
static __device__ __noinline__ double rcp_library(double x) { return 1.0 / x; }
static __device__ __noinline__ double rsqrt_library(double x) { return rsqrt(x); }

// e^x for -700 <= x <= 0 by Tang's table-driven method (P. T. P. Tang, ACM TOMS 15(2),
// 144-157, 1989), in base 2 with 256 table entries: x = (256 m + j) ln2/256 + r with
// |r| <= ln2/512, e^x = 2^m * 2^(j/256) * (1 + p(r)), p the degree-4 Taylor polynomial of
// e^r - 1 (truncation error below 4e-17 relative).  9 FP64 instructions.  The result lies
// in [2^-1011, 1] (normal), so 2^m is applied by an integer add to its exponent field.
__device__ __forceinline__ double exp_nonpos(double x, const double *tab) {
    const unsigned hi = (unsigned)__double2hiint(x);
    // sign set and |x| <= 700 (the high word of -700.0 is 0xC085E000); -0.0 included
    if (!(hi >= 0x80000000u && hi <= 0xC085E000u)) return exp_library(x);
    const double z = fma(x, kInvLn2xN, kRoundShifter);
    const int k = __double2loint(z);  // round(256 x / ln2), two's complement in the low word
    const double kd = z - kRoundShifter;
    double r = fma(kd, -kLn2HiD, x);
    r = fma(kd, -kLn2LoD, r);
    double c = fma(r, 1.0 / 24.0, 1.0 / 6.0);
    c = fma(c, r, 0.5);
    c = fma(c, r, 1.0);
    const double tj = tab[k & (kExp64N - 1)];
    const double y = fma(tj, c * r, tj);
    const int m = k >> kExp64Bits;  // floor(k / 256) (arithmetic shift)
    return __hiloint2double(__double2hiint(y) + m * (1 << 20), __double2loint(y));
}

// 1/x from the hardware approximation (rcp.approx.ftz.f64, relative error e0 well below
// 2^-20) and one cubically convergent Newton correction r (1 + h + h^2), h = 1 - x r:
// relative error O(e0^3) plus rounding.  3 FP64 instructions.  For x and 1/x normal.
__device__ __forceinline__ double rcp_normal(double x) {
    const unsigned e = ((unsigned)__double2hiint(x) >> 20) & 0x7ffu;
    if (e < 2u || e > 2044u) return rcp_library(x);
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    const double h = fma(-x, r, 1.0);
    return fma(r, fma(h, h, h), r);
}

// 1/sqrt(x) from the hardware approximation (rsqrt.approx.ftz.f64) and one cubically
// convergent correction y (1 + h/2 + 3h^2/8), h = 1 - x y^2.  5 FP64 instructions.  For
// positive normal x.
__device__ __forceinline__ double rsqrt_normal(double x) {
    const unsigned e = (unsigned)__double2hiint(x) >> 20;  // sign bit included
    if (e < 2u || e > 2044u) return rsqrt_library(x);
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double h = fma(-x * y, y, 1.0);
    const double c = fma(h, 0.375, 0.5);
    return fma(y * h, c, y);
}

}  // namespace pnjl
