// tt_metric.cuh — device Minkowski kernels that reproduce the reference's
// float32 results bit for bit.
//
// The reference (metric.hpp:92-207) evaluates each distance with 8-wide SIMD
// accumulators and a fixed horizontal reduction. IEEE-754 single precision
// with round-to-nearest gives the same bits on any hardware as long as every
// operation is the same operation in the same order, so each function below
// replays the reference's lane order with explicit __fadd_rn / __fmaf_rn /
// __fsqrt_rn (no contraction or reassociation is possible through these
// intrinsics).
#pragma once
#include "tt_common.cuh"
#include "tt_libm.cuh"

namespace tt {

enum MetricKind : int { M_L1 = 0, M_L2 = 1, M_LINF = 2, M_LP = 3 };

__device__ __forceinline__ f32 hsum8(const f32 t[8]) {
    // metric.hpp:33-37: ((t0+t1)+(t2+t3))+((t4+t5)+(t6+t7))
    return __fadd_rn(__fadd_rn(__fadd_rn(t[0], t[1]), __fadd_rn(t[2], t[3])),
                     __fadd_rn(__fadd_rn(t[4], t[5]), __fadd_rn(t[6], t[7])));
}

// kern::l2 (metric.hpp:92-112). dim >= 16: lane l of acc0 sums coordinates
// k = 16c + l, lane l of acc1 sums k = 16c + 8 + l (one fma per chunk c, in
// chunk order), then hsum8(acc0 + acc1); the scalar tail continues with fma
// from that sum; dim < 16 is one fma chain from 0. A generic accessor lets
// the same code read points from global or shared memory.
template <typename A, typename B>
__device__ __forceinline__ f32 l2_sq_acc(const A& a, const B& b, u32 dim) {
    u32 k = 0;
    f32 s = 0.0f;
    if (dim >= 16) {
        const u32 chunks = dim >> 4;
        f32 t[8];
#pragma unroll
        for (int l = 0; l < 8; ++l) {
            f32 a0 = 0.0f, a1 = 0.0f;
#pragma unroll
            for (u32 c = 0; c < chunks; ++c) {
                const f32 d0 = __fsub_rn(a(16 * c + l), b(16 * c + l));
                const f32 d1 = __fsub_rn(a(16 * c + 8 + l), b(16 * c + 8 + l));
                a0 = __fmaf_rn(d0, d0, a0);
                a1 = __fmaf_rn(d1, d1, a1);
            }
            t[l] = __fadd_rn(a0, a1);
        }
        s = hsum8(t);
        k = chunks << 4;
    }
#pragma unroll
    for (; k < dim; ++k) {
        const f32 d = __fsub_rn(a(k), b(k));
        s = __fmaf_rn(d, d, s);
    }
    return s;
}

// The reference's l2 is the IEEE square root of l2_sq_acc's sum.
template <typename A, typename B>
__device__ __forceinline__ f32 l2_acc(const A& a, const B& b, u32 dim) {
    return __fsqrt_rn(l2_sq_acc(a, b, dim));
}

// Every s >= 0 with sqrt_rn(s) <= d satisfies s <= sq_bound(d): sqrt(s) must
// lie below the next float above d, so s is below that float squared
// (rounded up). Lets a scan reject most candidates before the square root.
__device__ __forceinline__ f32 sq_bound(f32 d) {
    if (!(d < INFINITY)) return INFINITY;
    const f32 up = __uint_as_float(__float_as_uint(d) + 1u);
    return __fmul_ru(up, up);
}

// kern::l1 (metric.hpp:144-159).
template <typename A, typename B>
__device__ __forceinline__ f32 l1_acc(const A& a, const B& b, u32 dim) {
    u32 k = 0;
    f32 s = 0.0f;
    if (dim >= 16) {
        const u32 chunks = dim >> 4;
        f32 t[8];
#pragma unroll
        for (int l = 0; l < 8; ++l) {
            f32 a0 = 0.0f, a1 = 0.0f;
#pragma unroll
            for (u32 c = 0; c < chunks; ++c) {
                a0 = __fadd_rn(a0, fabsf(__fsub_rn(a(16 * c + l), b(16 * c + l))));
                a1 = __fadd_rn(a1, fabsf(__fsub_rn(a(16 * c + 8 + l), b(16 * c + 8 + l))));
            }
            t[l] = __fadd_rn(a0, a1);
        }
        s = hsum8(t);
        k = chunks << 4;
    }
#pragma unroll
    for (; k < dim; ++k) s = __fadd_rn(s, fabsf(__fsub_rn(a(k), b(k))));
    return s;
}

// kern::linf (metric.hpp:161-174): a max of |a_k - b_k|, order-free.
template <typename A, typename B>
__device__ __forceinline__ f32 linf_acc(const A& a, const B& b, u32 dim) {
    f32 m = 0.0f;
#pragma unroll
    for (u32 k = 0; k < dim; ++k) m = fmaxf(m, fabsf(__fsub_rn(a(k), b(k))));
    return m;
}

// kern::ipow (metric.hpp:176-181): square-and-multiply, same products.
__device__ __forceinline__ f32 ipow_dev(f32 x, u32 p) {
    f32 r = 1.0f;
    for (; p; p >>= 1, x = __fmul_rn(x, x))
        if (p & 1) r = __fmul_rn(r, x);
    return r;
}

// pow01_8 (metric.hpp:50-89), one lane: x^p for x in [0, 1] via
// exp2(p * log2 x) with the reference's series and constants, as the
// reference runs it on an aarch64 host: rcp_ps is FRECPE plus one FRECPS
// step (tt_libm.cuh), and GCC's default contraction fuses the two
// multiply-adds that SIMDe leaves as separate operations (the fnmadd of the
// Newton step, written -(a*b) + c, and lg = (e - 127) + S * 2.885...).
__device__ __forceinline__ f32 pow01_dev(f32 x, f32 p) {
    const u32 xi = __float_as_uint(x);
    const f32 e = __int2float_rn(int((xi & 0x7f800000u) >> 23));
    const f32 m = __uint_as_float((xi & 0x007fffffu) | 0x3f800000u);
    const f32 m1 = __fadd_rn(m, 1.0f);
    f32 r = rcp_a64_2to3(m1);
    r = __fmul_rn(r, __fmaf_rn(-m1, r, 2.0f));
    const f32 t = __fmul_rn(__fsub_rn(m, 1.0f), r);
    const f32 t2 = __fmul_rn(t, t);
    f32 S = 1.0f / 13.0f;
    S = __fmaf_rn(t2, S, 1.0f / 11.0f);
    S = __fmaf_rn(t2, S, 1.0f / 9.0f);
    S = __fmaf_rn(t2, S, 1.0f / 7.0f);
    S = __fmaf_rn(t2, S, 1.0f / 5.0f);
    S = __fmaf_rn(t2, S, 1.0f / 3.0f);
    S = __fmaf_rn(t2, S, 1.0f);
    S = __fmul_rn(S, t);
    const f32 lg = __fmaf_rn(S, 2.885390081777927f, __fsub_rn(e, 127.0f));
    const f32 y = fmaxf(__fmul_rn(p, lg), -126.0f);
    const f32 k = rintf(y);
    const f32 f = __fmul_rn(__fsub_rn(y, k), 0.6931471805599453f);
    f32 P = 1.0f / 720.0f;
    P = __fmaf_rn(f, P, 1.0f / 120.0f);
    P = __fmaf_rn(f, P, 1.0f / 24.0f);
    P = __fmaf_rn(f, P, 1.0f / 6.0f);
    P = __fmaf_rn(f, P, 0.5f);
    P = __fmaf_rn(f, P, 1.0f);
    P = __fmaf_rn(f, P, 1.0f);
    const u32 pb = __float_as_uint(P) + (u32(__float2int_rn(k)) << 23);
    return x < 1e-30f ? 0.0f : __uint_as_float(pb);
}

// The scalar std::pow(float, float) calls of kern::lp: glibc's powf.
__device__ __forceinline__ f32 powf_dev(f32 x, f32 y) { return powf_a64(x, y); }

// kern::lp (metric.hpp:183-207) up to its final root: M = max |a_k - b_k|
// and the sum s of (|a_k - b_k| / M)^p; the distance is M * powf(s, 1/p)
// (0 when M == 0).
template <typename A, typename B>
__device__ __forceinline__ void lp_parts(const A& a, const B& b, u32 dim, f32 p, f32& M, f32& s) {
    M = linf_acc(a, b, dim);
    s = 0.0f;
    if (M == 0.0f) return;
    const f32 inv = __fdiv_rn(1.0f, M);
    const bool integral = p == floorf(p) && p <= 8.0f;
    u32 k = 0;
    if (!integral && dim >= 8) {
        f32 acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (; k + 8 <= dim; k += 8)
#pragma unroll
            for (int l = 0; l < 8; ++l)
                acc[l] = __fadd_rn(acc[l], pow01_dev(fminf(__fmul_rn(fabsf(__fsub_rn(a(k + l), b(k + l))), inv), 1.0f), p));
        s = hsum8(acc);
    }
    for (; k < dim; ++k) {
        const f32 x = fminf(1.0f, __fmul_rn(fabsf(__fsub_rn(a(k), b(k))), inv));
        s = __fadd_rn(s, integral ? ipow_dev(x, u32(p)) : powf_dev(x, p));
    }
}

__device__ __forceinline__ f32 lp_root(f32 M, f32 s, f32 p) {
    return M == 0.0f ? 0.0f : __fmul_rn(M, powf_dev(s, __fdiv_rn(1.0f, p)));
}

// A lower bound of lp_root(M, s, p) from float arithmetic: powf's result is
// within 1 ulp of s^(1/p), and the fast exp2/log2 path errs by far less than
// the 2^-14 relative margin taken here, so a candidate whose bound already
// exceeds a threshold cannot pass it (scans skip the exact root for it).
__device__ __forceinline__ f32 lp_root_lower(f32 M, f32 s, f32 p) {
    return __fmul_rd(__fmul_rd(M, __powf(s, __fdividef(1.0f, p))), 1.0f - 0x1p-14f);
}

// lp_parts for a caller that only needs distances up to `bound`: after each
// 8-coordinate chunk but the last it stops, returning false, once the sum so
// far already puts the distance above bound. Every term is >= 0 and a float
// sum of non-negative terms never decreases, so the partial hsum8 is at most
// the final s, and lp_root_lower of it is a lower bound of the distance as
// much as of the final sum's root. Returns true with M and s exactly as
// lp_parts computes them otherwise.
template <typename A, typename B>
__device__ __forceinline__ bool lp_parts_within(const A& a, const B& b, u32 dim, f32 p, f32 bound, f32& M, f32& s) {
    M = linf_acc(a, b, dim);
    s = 0.0f;
    if (M == 0.0f) return true;
    const f32 inv = __fdiv_rn(1.0f, M);
    const bool integral = p == floorf(p) && p <= 8.0f;
    u32 k = 0;
    if (!integral && dim >= 8) {
        f32 acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (; k + 8 <= dim; k += 8) {
#pragma unroll
            for (int l = 0; l < 8; ++l)
                acc[l] = __fadd_rn(acc[l], pow01_dev(fminf(__fmul_rn(fabsf(__fsub_rn(a(k + l), b(k + l))), inv), 1.0f), p));
            if (k + 16 <= dim && lp_root_lower(M, hsum8(acc), p) > bound) return false;
        }
        s = hsum8(acc);
    }
    for (; k < dim; ++k) {
        const f32 x = fminf(1.0f, __fmul_rn(fabsf(__fsub_rn(a(k), b(k))), inv));
        s = __fadd_rn(s, integral ? ipow_dev(x, u32(p)) : powf_dev(x, p));
    }
    return true;
}

template <typename A, typename B>
__device__ __forceinline__ f32 lp_acc(const A& a, const B& b, u32 dim, f32 p) {
    f32 M, s;
    lp_parts(a, b, dim, p, M, s);
    return lp_root(M, s, p);
}

template <typename A, typename B>
__device__ __forceinline__ f32 metric_dist(int kind, f32 p, const A& a, const B& b, u32 dim) {
    switch (kind) {
        case M_L1: return l1_acc(a, b, dim);
        case M_L2: return l2_acc(a, b, dim);
        case M_LINF: return linf_acc(a, b, dim);
        default: return lp_acc(a, b, dim, p);
    }
}

// Row accessor over a contiguous float row (global or shared memory).
struct Row {
    const f32* p;
    __device__ __forceinline__ f32 operator()(u32 k) const { return p[k]; }
};

__device__ __forceinline__ f32 dist_rows(int kind, f32 p, const f32* a, const f32* b, u32 dim) {
    return metric_dist(kind, p, Row{a}, Row{b}, dim);
}

}  // namespace tt
