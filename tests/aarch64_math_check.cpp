// aarch64_math_check.cpp — pins the oracle's restatements in
// oracle/aarch64_math.h to the real thing on the host it runs on:
//
//   frecpe   every float, against the FRECPE instruction (aarch64 only)
//   rcp      every float in [1, 4), against SIMDe's NEON rcp sequence
//            vmulq(e, vrecpsq(e, a)) with e = vrecpeq(a) (aarch64 only)
//   powf     the host libm's powf over every x in [1, 32) with y = 1/1.5f (the
//            final root of an lp:1.5 distance in R^32), every x in [0, 1] with
//            y = 1.5f and y = 2.5f (the scalar terms of short vectors), and
//            seeded random (x, y) pairs of both signs and all exponents
//
// Prints one line per check: "<name> <tested> <mismatches> [first mismatch]".
// Built by tests/test_aarch64_math.py with -ffp-contract=off so only the
// restatement's explicit fma calls fuse.
#include "aarch64_math.h"

#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <thread>
#include <vector>
#if defined(__aarch64__)
#include <arm_neon.h>
#endif

using namespace a64;

namespace {

#if defined(__aarch64__)
constexpr bool kTiesAway = true;
#else
constexpr bool kTiesAway = false;
#endif

struct Result {
    std::atomic<uint64_t> tested{0}, bad{0};
    std::atomic<uint64_t> first{~uint64_t(0)};
    void mismatch(uint64_t key) {
        bad.fetch_add(1);
        uint64_t cur = first.load();
        while (key < cur && !first.compare_exchange_weak(cur, key)) {}
    }
};

template <typename F>
void parallel(uint64_t lo, uint64_t hi, F&& f) {
    const unsigned nt = std::max(1u, std::thread::hardware_concurrency());
    std::vector<std::thread> th;
    const uint64_t chunk = (hi - lo + nt - 1) / nt;
    for (unsigned t = 0; t < nt; ++t) {
        const uint64_t a = lo + t * chunk, b = std::min(hi, a + chunk);
        if (a >= b) break;
        th.emplace_back([=, &f] { f(a, b); });
    }
    for (auto& x : th) x.join();
}

bool same(float a, float b) { return fbits(a) == fbits(b) || (std::isnan(a) && std::isnan(b)); }

void report(const char* name, Result& r, const char* detail = "") {
    std::printf("%s %llu %llu %s\n", name, (unsigned long long)r.tested.load(),
                (unsigned long long)r.bad.load(), r.bad.load() ? detail : "");
}

void check_pow_range(const char* name, float lo, float hi, float y) {
    Result r;
    const uint32_t a = fbits(lo), b = fbits(hi);
    parallel(a, b, [&](uint64_t s, uint64_t e) {
        uint64_t bad = 0;
        for (uint64_t u = s; u < e; ++u) {
            const float x = bitsf(uint32_t(u));
            if (!same(ref_powf(x, y, kTiesAway), powf(x, y))) { ++bad; r.mismatch(u); }
        }
        r.tested.fetch_add(e - s);
        (void)bad;
    });
    char buf[128] = "";
    if (r.bad.load()) {
        const float x = bitsf(uint32_t(r.first.load()));
        std::snprintf(buf, sizeof buf, "x=%a y=%a ref=%a libm=%a", x, y, ref_powf(x, y, kTiesAway), powf(x, y));
    }
    report(name, r, buf);
}

}  // namespace

int main(int argc, char** argv) {
    const bool quick = argc > 1 && std::string(argv[1]) == "quick";
#if defined(__aarch64__)
    {
        Result r;
        parallel(0, uint64_t(1) << 32, [&](uint64_t s, uint64_t e) {
            for (uint64_t u = s; u < e; ++u) {
                const float x = bitsf(uint32_t(u));
                if (!same(frecpe(x), vrecpes_f32(x))) r.mismatch(u);
            }
            r.tested.fetch_add(e - s);
        });
        char buf[96] = "";
        if (r.bad.load()) {
            const float x = bitsf(uint32_t(r.first.load()));
            std::snprintf(buf, sizeof buf, "x=%a ours=%a hw=%a", x, frecpe(x), vrecpes_f32(x));
        }
        report("frecpe", r, buf);
    }
    {
        Result r;
        parallel(fbits(1.0f), fbits(4.0f), [&](uint64_t s, uint64_t e) {
            for (uint64_t u = s; u < e; ++u) {
                const float x = bitsf(uint32_t(u));
                const float32x4_t a = vdupq_n_f32(x);
                float32x4_t rc = vrecpeq_f32(a);
                rc = vmulq_f32(rc, vrecpsq_f32(rc, a));
                if (!same(rcp_ps(x), vgetq_lane_f32(rc, 0))) r.mismatch(u);
            }
            r.tested.fetch_add(e - s);
        });
        report("rcp", r);
    }
#else
    std::printf("frecpe skipped (not aarch64)\n");
#endif
    check_pow_range("powf_root_1.5", 1.0f, 32.0f, 1.0f / 1.5f);
    check_pow_range("powf_root_3.5", 1.0f, quick ? 2.0f : 32.0f, 1.0f / 3.5f);
    check_pow_range("powf_term_1.5", 0.0f, quick ? 0x1p-100f : 1.0f, 1.5f);
    check_pow_range("powf_term_1.5_top", 0.5f, 1.0f, 1.5f);
    check_pow_range("powf_term_2.5", quick ? 0.5f : 0.0f, 1.0f, 2.5f);
    {
        // random pairs: x over every exponent and sign, y from a few shapes
        Result r;
        const uint64_t total = quick ? (uint64_t(1) << 22) : (uint64_t(1) << 27);
        parallel(0, total, [&](uint64_t s, uint64_t e) {
            uint64_t st = 0x9e3779b97f4a7c15ull ^ (s * 0xbf58476d1ce4e5b9ull);
            auto next = [&] { st ^= st >> 12; st ^= st << 25; st ^= st >> 27; return st * 0x2545f4914f6cdd1dull; };
            for (uint64_t i = s; i < e; ++i) {
                const uint64_t v = next();
                const float x = bitsf(uint32_t(v));
                float y;
                switch ((v >> 32) & 3) {
                    case 0: y = bitsf(uint32_t(v >> 32) & 0x41ffffffu); break;           // |y| < 32
                    case 1: y = float(int((v >> 34) & 63) - 32); break;                    // integers
                    case 2: y = float(int((v >> 34) & 255) - 128) * 0.5f; break;           // halves
                    default: y = 1.0f / (1.0f + float((v >> 34) & 1023) / 64.0f); break;  // 1/p roots
                }
                if (!same(ref_powf(x, y, kTiesAway), powf(x, y))) r.mismatch(i);
            }
            r.tested.fetch_add(e - s);
        });
        report("powf_random", r);
    }
    return 0;
}
