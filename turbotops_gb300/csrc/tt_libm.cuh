// tt_libm.cuh — device replays of the host arithmetic that decides the
// reference's non-integer Lp distances (metric.hpp:50-89, :183-207) on the
// host it runs beside: the GB300 machine's Grace CPU (aarch64), where the
// reference's SIMD code runs through SIMDe 0.8.4's NEON translation and its
// scalar std::pow(float, float) calls are glibc's powf.
//
//  * simde_mm256_rcp_ps on NEON (third_party/simde/simde/x86/avx2.h:
//    15474-15490, SIMDE_ACCURACY_PREFERENCE 1) is FRECPE followed by one
//    FRECPS Newton step: e = FRECPE(a); e * (2 - e*a) with the inner step
//    fused. FRECPE is an architected table-free estimate: the Arm
//    Architecture Reference Manual's RecipEstimate takes the top 8 fraction
//    bits of a, a' = 2*(256 + bits) + 1, and returns the 8 fraction bits of
//    ((2^19 / a') + 1) / 2 (integer division) under the Linux default FPCR.
//  * glibc powf (sysdeps/ieee754/flt-32/e_powf.c since glibc 2.28, from Arm's
//    optimized-routines): x^y = exp2(y * log2 x) in double precision. log2 x
//    = k + log2 c + P(z/c - 1) with c from a 16-entry table picked by the top
//    bits of x - 0x3f330000 and P of degree 5; exp2 splits y*log2(x) into
//    m/32 + r (m rounded halfway away from zero, as the aarch64 port's
//    round()/lround() do), takes 2^(m/32) from a 32-entry table and 2^r from a
//    cubic, then rounds once to float. Every multiply-add is fused, as GCC's
//    default contraction compiles them.
//
// FP64 appears here only because the reference's libm computes in double:
// replaying its double-precision steps is what makes the final float round
// the same way. The scans call it only for candidates that a float-precision
// lower bound cannot reject.
#pragma once
#include "tt_common.cuh"

namespace tt {

// FRECPE(a) * FRECPS step, for a in [2, 3) (the m + 1 of pow01_8; every such
// a has biased exponent 128, so the estimate's exponent is 253 - 128 = 125).
__device__ __forceinline__ f32 rcp_a64_2to3(f32 a) {
    const u32 top8 = (__float_as_uint(a) >> 15) & 0xffu;
    const int den = 2 * int(256u | top8) + 1;                 // 513 .. 1023, odd
    // floor(2^19 / den): the quotient is never within 1/1023 of an integer,
    // far more than the 2-ulp error of the fast division near 1000 (2^-13).
    const int b = int(__fdividef(524288.0f, float(den)));
    const u32 r = u32((b + 1) >> 1) & 0xffu;
    const f32 e = __uint_as_float((125u << 23) | (r << 15));
    return __fmul_rn(e, __fmaf_rn(-e, a, 2.0f));
}

__device__ const double kPowfInvc[16] = {
    0x1.661ec79f8f3bep+0, 0x1.571ed4aaf883dp+0, 0x1.49539f0f010bp+0, 0x1.3c995b0b80385p+0,
    0x1.30d190c8864a5p+0, 0x1.25e227b0b8eap+0,  0x1.1bb4a4a1a343fp+0, 0x1.12358f08ae5bap+0,
    0x1.0953f419900a7p+0, 0x1p+0,               0x1.e608cfd9a47acp-1, 0x1.ca4b31f026aap-1,
    0x1.b2036576afce6p-1, 0x1.9c2d163a1aa2dp-1, 0x1.886e6037841edp-1, 0x1.767dcf5534862p-1};
__device__ const double kPowfLogc[16] = {
    -0x1.efec65b963019p-2, -0x1.b0b6832d4fca4p-2, -0x1.7418b0a1fb77bp-2, -0x1.39de91a6dcf7bp-2,
    -0x1.01d9bf3f2b631p-2, -0x1.97c1d1b3b7afp-3,  -0x1.2f9e393af3c9fp-3, -0x1.960cbbf788d5cp-4,
    -0x1.a6f9db6475fcep-5, 0x0p+0,                0x1.338ca9f24f53dp-4,  0x1.476a9543891bap-3,
    0x1.e840b4ac4e4d2p-3,  0x1.40645f0c6651cp-2,  0x1.88e9c2c1b9ff8p-2,  0x1.ce0a44eb17bccp-2};
// bits of 2^(i/32) minus i << 47
__device__ const unsigned long long kExp2Tab[32] = {
    0x3ff0000000000000ull, 0x3fefd9b0d3158574ull, 0x3fefb5586cf9890full, 0x3fef9301d0125b51ull,
    0x3fef72b83c7d517bull, 0x3fef54873168b9aaull, 0x3fef387a6e756238ull, 0x3fef1e9df51fdee1ull,
    0x3fef06fe0a31b715ull, 0x3feef1a7373aa9cbull, 0x3feedea64c123422ull, 0x3feece086061892dull,
    0x3feebfdad5362a27ull, 0x3feeb42b569d4f82ull, 0x3feeab07dd485429ull, 0x3feea47eb03a5585ull,
    0x3feea09e667f3bcdull, 0x3fee9f75e8ec5f74ull, 0x3feea11473eb0187ull, 0x3feea589994cce13ull,
    0x3feeace5422aa0dbull, 0x3feeb737b0cdc5e5ull, 0x3feec49182a3f090ull, 0x3feed503b23e255dull,
    0x3feee89f995ad3adull, 0x3feeff76f2fb5e47ull, 0x3fef199bdd85529cull, 0x3fef3720dcef9069ull,
    0x3fef5818dcfba487ull, 0x3fef7c97337b9b5full, 0x3fefa4afa2a490daull, 0x3fefd0765b6e4540ull};

// glibc powf for x >= 0 (every x an Lp distance feeds it: |d_k|/M in [0, 1]
// and the sum s in [1, dim]); y finite and nonzero.
static __device__ __noinline__ f32 powf_a64(f32 x, f32 y) {
    u32 ix = __float_as_uint(x);
    if (ix == 0u) return y > 0.0f ? 0.0f : INFINITY;            // +0^y
    if (ix == 0x3f800000u) return 1.0f;
    if (ix >= 0x7f800000u) return ix > 0x7f800000u ? x : (y > 0.0f ? INFINITY : 0.0f);
    if (ix < 0x00800000u) {                                        // subnormal: normalise
        ix = __float_as_uint(__fmul_rn(x, 0x1p23f)) - (23u << 23);
    }
    // log2(x) (e_powf.c log2_inline)
    const u32 tmp = ix - 0x3f330000u;
    const int i = int((tmp >> 19) & 15u);
    const u32 top = tmp & 0xff800000u;
    const u32 iz = ix - top;
    const int k = int(top) >> 23;
    const double z = double(__uint_as_float(iz));
    const double r = __fma_rn(z, kPowfInvc[i], -1.0);
    const double y0 = __dadd_rn(kPowfLogc[i], double(k));
    const double r2 = __dmul_rn(r, r);
    double q = __fma_rn(0x1.27616c9496e0bp-2, r, -0x1.71969a075c67ap-2);
    const double pp = __fma_rn(0x1.ec70a6ca7baddp-2, r, -0x1.7154748bef6c8p-1);
    const double r4 = __dmul_rn(r2, r2);
    double qq = __fma_rn(0x1.71547652ab82bp0, r, y0);
    qq = __fma_rn(pp, r2, qq);
    const double logx = __fma_rn(q, r4, qq);
    const double ylogx = __dmul_rn(double(y), logx);
    // range checks (|y log2 x| >= 126)
    if (((__double_as_longlong(ylogx) >> 47) & 0xffff) >= (__double_as_longlong(126.0) >> 47)) {
        if (ylogx > 0x1.fffffffd1d571p+6) return INFINITY;
        if (ylogx <= -150.0) return 0.0f;
        if (ylogx < -149.0) return 0x1p-149f;
    }
    // exp2 (e_powf.c exp2_inline, round()/lround() variant)
    const double kd = round(__dmul_rn(ylogx, 32.0));
    const unsigned long long ki = (unsigned long long)(long long)kd;
    const double rr = __dadd_rn(ylogx, -__dmul_rn(kd, 0.03125));
    unsigned long long t = kExp2Tab[ki & 31];
    t += ki << 47;
    const double s = __longlong_as_double((long long)t);
    const double zz = __fma_rn(0x1.c6af84b912394p-5, rr, 0x1.ebfce50fac4f3p-3);
    const double rr2 = __dmul_rn(rr, rr);
    double yy = __fma_rn(0x1.62e42ff0c52d6p-1, rr, 1.0);
    yy = __fma_rn(zz, rr2, yy);
    yy = __dmul_rn(yy, s);
    return __double2float_rn(yy);
}

}  // namespace tt
