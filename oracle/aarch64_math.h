// aarch64_math.h — test infrastructure only (the checker, never the product).
//
// CPU restatements of the three pieces of host arithmetic that decide the
// reference's non-integer Lp distances on an aarch64 host (the GB300 machine's
// Grace CPU), where the reference's SIMD code runs through SIMDe 0.8.4's NEON
// translation and its scalar pow calls go to glibc:
//
//   a64_frecpe   FRECPE, the Arm reciprocal estimate, single precision, as the
//                Arm Architecture Reference Manual's FPRecipEstimate /
//                RecipEstimate pseudo-code defines it under the Linux default
//                FPCR (FZ = 0, DN = 0, AH = 0: no FEAT_RPRES increased
//                precision), round to nearest.
//   a64_frecps   FRECPS, the fused Newton step 2 - a*b (FPRecipStepFused).
//   a64_rcp_ps   SIMDe's simde_mm_rcp_ps on NEON with its default
//                SIMDE_ACCURACY_PREFERENCE of 1 (third_party/simde/simde/x86/
//                avx2.h:15474-15490): e = FRECPE(a); e * FRECPS(e, a).
//   ref_powf     glibc's powf (sysdeps/ieee754/flt-32/e_powf.c since glibc
//                2.28, from Arm's optimized-routines, Szabolcs Nagy 2017-2018):
//                x^y = exp2(y * log2 x) evaluated in double — log2 from a
//                16-entry table of (1/c, log2 c) around which a degree-5
//                polynomial in r = z/c - 1 is evaluated, exp2 from a 32-entry
//                table of 2^(i/32) and a degree-3 polynomial — then one
//                rounding to float. The multiply-adds are fused as GCC
//                contracts them (default -ffp-contract=fast). `ties_away`
//                selects how the exp2 step rounds y*log2(x) to a multiple of
//                1/32: to even (the portable shift trick, x86-64) or away
//                from zero (round()/lround(), the TOINT_INTRINSICS variant
//                that glibc's aarch64 port enables); the two differ only when
//                y*log2(x) lies exactly halfway.
//
// These are checked against the hardware instruction (aarch64 only) and the
// host libm's powf by tests/test_aarch64_math.py.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace a64 {

inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float bitsf(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
inline uint64_t dbits(double d) { uint64_t u; std::memcpy(&u, &d, 8); return u; }
inline double bitsd(uint64_t u) { double d; std::memcpy(&d, &u, 8); return d; }

// FPRecipEstimate, N = 32.
inline float frecpe(float x) {
    const uint32_t u = fbits(x);
    const uint32_t sign = u & 0x80000000u;
    const uint32_t ex = (u >> 23) & 0xffu;
    const uint32_t fr = u & 0x7fffffu;
    if (ex == 0xffu) {
        if (fr) return bitsf(u | 0x400000u);        // NaN: quieted
        return bitsf(sign);                          // +-inf -> +-0
    }
    if (ex == 0 && fr == 0) return bitsf(sign | 0x7f800000u);   // +-0 -> +-inf
    if (ex == 0 && fr < 0x200000u) return bitsf(sign | 0x7f800000u);  // |x| < 2^-128: overflow, RN -> inf
    uint64_t f = uint64_t(fr) << 29;                 // 52-bit fraction
    int e = int(ex);
    const uint64_t m52 = (uint64_t(1) << 52) - 1;
    if (e == 0) {
        if (!((f >> 51) & 1)) { e = -1; f = (f << 2) & m52; }
        else f = (f << 1) & m52;
    }
    const int scaled = 256 | int(f >> 44);           // '1' : fraction<51:44>, 256..511
    int rexp = 253 - e;
    const int a = scaled * 2 + 1;
    const int b = (1 << 19) / a;
    const int r = (b + 1) / 2;                       // 256..511
    uint64_t rf = uint64_t(r & 0xff) << 44;
    if (rexp == 0) rf = (uint64_t(1) << 51) | (rf >> 1);
    else if (rexp == -1) { rf = (uint64_t(1) << 50) | (rf >> 2); rexp = 0; }
    return bitsf(sign | (uint32_t(rexp) << 23) | uint32_t(rf >> 29));
}

// FPRecipStepFused: 2 - a*b with one rounding; 0 * inf gives 2.
inline float frecps(float a, float b) {
    if (std::isnan(a) || std::isnan(b)) return a + b;
    if ((std::isinf(a) && b == 0.0f) || (a == 0.0f && std::isinf(b))) return 2.0f;
    return std::fma(-a, b, 2.0f);
}

inline float rcp_ps(float a) {
    const float e = frecpe(a);
    return e * frecps(e, a);
}

// ---- glibc powf ------------------------------------------------------------
struct PowfLog2Entry { double invc, logc; };
// (1/c, log2 c) for the 16 subintervals of [0x1.66p-1, 0x1.66p0) that the top
// bits of x - 0x3f330000 select.
inline constexpr PowfLog2Entry kPowfLog2[16] = {
    {0x1.661ec79f8f3bep+0, -0x1.efec65b963019p-2}, {0x1.571ed4aaf883dp+0, -0x1.b0b6832d4fca4p-2},
    {0x1.49539f0f010bp+0, -0x1.7418b0a1fb77bp-2},  {0x1.3c995b0b80385p+0, -0x1.39de91a6dcf7bp-2},
    {0x1.30d190c8864a5p+0, -0x1.01d9bf3f2b631p-2}, {0x1.25e227b0b8eap+0, -0x1.97c1d1b3b7afp-3},
    {0x1.1bb4a4a1a343fp+0, -0x1.2f9e393af3c9fp-3}, {0x1.12358f08ae5bap+0, -0x1.960cbbf788d5cp-4},
    {0x1.0953f419900a7p+0, -0x1.a6f9db6475fcep-5}, {0x1p+0, 0x0p+0},
    {0x1.e608cfd9a47acp-1, 0x1.338ca9f24f53dp-4},  {0x1.ca4b31f026aap-1, 0x1.476a9543891bap-3},
    {0x1.b2036576afce6p-1, 0x1.e840b4ac4e4d2p-3}, {0x1.9c2d163a1aa2dp-1, 0x1.40645f0c6651cp-2},
    {0x1.886e6037841edp-1, 0x1.88e9c2c1b9ff8p-2}, {0x1.767dcf5534862p-1, 0x1.ce0a44eb17bccp-2},
};
// log2(1 + r) ~ A0 r^5 + A1 r^4 + A2 r^3 + A3 r^2 + A4 r
inline constexpr double kPowfA[5] = {0x1.27616c9496e0bp-2, -0x1.71969a075c67ap-2, 0x1.ec70a6ca7baddp-2,
                                     -0x1.7154748bef6c8p-1, 0x1.71547652ab82bp0};
// bits of 2^(i/32) (nearest double) minus i << 47, so that adding k << 47 for
// k = 32 m + i scales by 2^m.
inline constexpr uint64_t kExp2T[32] = {
    0x3ff0000000000000, 0x3fefd9b0d3158574, 0x3fefb5586cf9890f, 0x3fef9301d0125b51, 0x3fef72b83c7d517b,
    0x3fef54873168b9aa, 0x3fef387a6e756238, 0x3fef1e9df51fdee1, 0x3fef06fe0a31b715, 0x3feef1a7373aa9cb,
    0x3feedea64c123422, 0x3feece086061892d, 0x3feebfdad5362a27, 0x3feeb42b569d4f82, 0x3feeab07dd485429,
    0x3feea47eb03a5585, 0x3feea09e667f3bcd, 0x3fee9f75e8ec5f74, 0x3feea11473eb0187, 0x3feea589994cce13,
    0x3feeace5422aa0db, 0x3feeb737b0cdc5e5, 0x3feec49182a3f090, 0x3feed503b23e255d, 0x3feee89f995ad3ad,
    0x3feeff76f2fb5e47, 0x3fef199bdd85529c, 0x3fef3720dcef9069, 0x3fef5818dcfba487, 0x3fef7c97337b9b5f,
    0x3fefa4afa2a490da, 0x3fefd0765b6e4540,
};
// 2^r ~ 1 + C2 r + C1 r^2 + C0 r^3, |r| <= 1/64
inline constexpr double kExp2C[3] = {0x1.c6af84b912394p-5, 0x1.ebfce50fac4f3p-3, 0x1.62e42ff0c52d6p-1};

inline double powf_log2(uint32_t ix) {
    const uint32_t tmp = ix - 0x3f330000u;
    const int i = int((tmp >> 19) % 16);
    const uint32_t top = tmp & 0xff800000u;
    const uint32_t iz = ix - top;
    const int k = int32_t(top) >> 23;
    const double invc = kPowfLog2[i].invc, logc = kPowfLog2[i].logc;
    const double z = double(bitsf(iz));
    const double r = std::fma(z, invc, -1.0);
    const double y0 = logc + double(k);
    const double r2 = r * r;
    double y = std::fma(kPowfA[0], r, kPowfA[1]);
    const double p = std::fma(kPowfA[2], r, kPowfA[3]);
    const double r4 = r2 * r2;
    double q = std::fma(kPowfA[4], r, y0);
    q = std::fma(p, r2, q);
    y = std::fma(y, r4, q);
    return y;
}

inline float powf_exp2(double xd, uint64_t sign_bias, bool ties_away) {
    double kd;
    uint64_t ki;
    if (ties_away) {
        // 32 * xd to the nearest integer, halfway away from zero
        const double xs = xd * 32.0;
        kd = std::round(xs);
        ki = uint64_t(int64_t(kd));
        kd = kd / 32.0;
    } else {
        const double shift = 0x1.8p+47;
        kd = xd + shift;
        ki = dbits(kd);
        kd -= shift;
    }
    const double r = xd - kd;
    uint64_t t = kExp2T[ki % 32];
    const uint64_t ski = ki + sign_bias;
    t += ski << 47;
    const double s = bitsd(t);
    const double z = std::fma(kExp2C[0], r, kExp2C[1]);
    const double r2 = r * r;
    double y = std::fma(kExp2C[2], r, 1.0);
    y = std::fma(z, r2, y);
    y = y * s;
    return float(y);
}

inline int powf_checkint(uint32_t iy) {
    const int e = int(iy >> 23 & 0xff);
    if (e < 0x7f) return 0;
    if (e > 0x7f + 23) return 2;
    if (iy & ((1u << (0x7f + 23 - e)) - 1)) return 0;
    if (iy & (1u << (0x7f + 23 - e))) return 1;
    return 2;
}

inline bool powf_signaling(uint32_t ix) { return 2 * (ix ^ 0x00400000u) > 2u * 0x7fc00000u; }

inline bool powf_zeroinfnan(uint32_t ix) { return 2 * ix - 1 >= 2u * 0x7f800000u - 1; }

inline float ref_powf(float x, float y, bool ties_away) {
    uint64_t sign_bias = 0;
    uint32_t ix = fbits(x);
    const uint32_t iy = fbits(y);
    if (ix - 0x00800000u >= 0x7f800000u - 0x00800000u || powf_zeroinfnan(iy)) {
        if (powf_zeroinfnan(iy)) {
            if (2 * iy == 0) return powf_signaling(ix) ? x + y : 1.0f;
            if (ix == 0x3f800000u) return powf_signaling(iy) ? x + y : 1.0f;
            if (2 * ix > 2u * 0x7f800000u || 2 * iy > 2u * 0x7f800000u) return x + y;
            if (2 * ix == 2 * 0x3f800000u) return 1.0f;
            if ((2 * ix < 2 * 0x3f800000u) == !(iy & 0x80000000u)) return 0.0f;
            return y * y;
        }
        if (powf_zeroinfnan(ix)) {
            float x2 = x * x;
            if ((ix & 0x80000000u) && powf_checkint(iy) == 1) x2 = -x2;
            return (iy & 0x80000000u) ? 1.0f / x2 : x2;
        }
        if (ix & 0x80000000u) {
            const int yint = powf_checkint(iy);
            if (yint == 0) return std::nanf("");
            if (yint == 1) sign_bias = uint64_t(1) << 16;
            ix &= 0x7fffffffu;
        }
        if (ix < 0x00800000u) {
            ix = fbits(bitsf(ix) * 0x1p23f);
            ix &= 0x7fffffffu;
            ix -= 23u << 23;
        }
    }
    const double logx = powf_log2(ix);
    const double ylogx = double(y) * logx;
    if ((dbits(ylogx) >> 47 & 0xffff) >= dbits(126.0) >> 47) {
        if (ylogx > 0x1.fffffffd1d571p+6) return sign_bias ? -INFINITY : INFINITY;
        if (ylogx <= -150.0) return sign_bias ? -0.0f : 0.0f;
        if (ylogx < -149.0) return sign_bias ? -0x1p-149f : 0x1p-149f;
    }
    return powf_exp2(ylogx, sign_bias, ties_away);
}

}  // namespace a64
