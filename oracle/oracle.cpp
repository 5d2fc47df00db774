// oracle.cpp — TEST INFRASTRUCTURE ONLY: scalar CPU restatement of the
// reference's front end (dnbaker/turbotops v0.1.0). Only tests/ and bench.py's
// CPU leg load it, as the checker. Compiled with -ffp-contract=off: every fused
// multiply-add below is an explicit fmaf where the reference fuses.
#include "oracle.h"
#include "aarch64_math.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>
#include <thread>
#include <vector>

namespace {

using u8 = uint8_t;
using u32 = uint32_t;
using u64 = uint64_t;
using f32 = float;
constexpr u64 kNone = ~0ull;

// ---------------------------------------------------------------------------
// Metrics (metric.hpp:33-207)
// ---------------------------------------------------------------------------
// hsum8 (metric.hpp:33-37): ((t0+t1)+(t2+t3))+((t4+t5)+(t6+t7)).
f32 hsum8(const f32* t) { return ((t[0] + t[1]) + (t[2] + t[3])) + ((t[4] + t[5]) + (t[6] + t[7])); }

// kern::l2 (metric.hpp:92-112). dim >= 16: lanes k%16 in [0,8) accumulate in
// acc0 and [8,16) in acc1 with one fma per 16-chunk; hsum8(acc0 + acc1); then a
// scalar fma tail; then sqrt.
f32 l2(const f32* a, const f32* b, u32 dim) {
    u32 k = 0;
    f32 s = 0.0f;
    if (dim >= 16) {
        f32 acc0[8] = {0}, acc1[8] = {0};
        for (; k + 16 <= dim; k += 16)
            for (int l = 0; l < 8; ++l) {
                const f32 d0 = a[k + l] - b[k + l], d1 = a[k + 8 + l] - b[k + 8 + l];
                acc0[l] = std::fmaf(d0, d0, acc0[l]);
                acc1[l] = std::fmaf(d1, d1, acc1[l]);
            }
        f32 t[8];
        for (int l = 0; l < 8; ++l) t[l] = acc0[l] + acc1[l];
        s = hsum8(t);
    }
    for (; k < dim; ++k) {
        const f32 d = a[k] - b[k];
        s = std::fmaf(d, d, s);
    }
    return std::sqrt(s);
}

// kern::l1 (metric.hpp:144-159).
f32 l1(const f32* a, const f32* b, u32 dim) {
    u32 k = 0;
    f32 s = 0.0f;
    if (dim >= 16) {
        f32 acc0[8] = {0}, acc1[8] = {0};
        for (; k + 16 <= dim; k += 16)
            for (int l = 0; l < 8; ++l) {
                acc0[l] = acc0[l] + std::fabs(a[k + l] - b[k + l]);
                acc1[l] = acc1[l] + std::fabs(a[k + 8 + l] - b[k + 8 + l]);
            }
        f32 t[8];
        for (int l = 0; l < 8; ++l) t[l] = acc0[l] + acc1[l];
        s = hsum8(t);
    }
    for (; k < dim; ++k) s += std::fabs(a[k] - b[k]);
    return s;
}

// kern::linf (metric.hpp:161-174): a max, so the lane order is immaterial.
f32 linf(const f32* a, const f32* b, u32 dim) {
    f32 m = 0.0f;
    for (u32 k = 0; k < dim; ++k) m = std::max(m, std::fabs(a[k] - b[k]));
    return m;
}

// kern::ipow (metric.hpp:176-181).
f32 ipow(f32 x, u32 p) {
    f32 r = 1.0f;
    for (; p; p >>= 1, x *= x)
        if (p & 1) r *= x;
    return r;
}

// The Lp model: the reference's non-integer-p arithmetic as it runs on an
// aarch64 host (SIMDe's NEON translation, glibc powf), aarch64_math.h.
// Bits of g_lp_model select where GCC's default contraction (-ffp-contract=
// fast) fuses a multiply into the following add; the default is the one that
// reproduces the reference built on the GB300 machine's Grace host.
//   bit 0  SIMDe's portable fnmadd, -(a*b) + c, fused (rcp refinement)
//   bit 1  lg = (e - 127) + S * 2.885..., fused
//   bit 2  glibc powf rounds y*log2(x) halfway away from zero (aarch64 port)
int g_lp_model = 7;

// pow01_8 (metric.hpp:50-89), one lane.
f32 pow01(f32 x, f32 p) {
    u32 xi;
    std::memcpy(&xi, &x, 4);
    const f32 e = f32(int32_t((xi & 0x7f800000u) >> 23));
    const u32 mi = (xi & 0x007fffffu) | 0x3f800000u;
    f32 m;
    std::memcpy(&m, &mi, 4);
    const f32 m1 = m + 1.0f;
    f32 r = a64::rcp_ps(m1);
    const f32 nm = (g_lp_model & 1) ? std::fmaf(-m1, r, 2.0f) : -(m1 * r) + 2.0f;
    r = r * nm;
    const f32 t = (m - 1.0f) * r;
    const f32 t2 = t * t;
    f32 S = 1.0f / 13.0f;
    S = std::fmaf(t2, S, 1.0f / 11.0f);
    S = std::fmaf(t2, S, 1.0f / 9.0f);
    S = std::fmaf(t2, S, 1.0f / 7.0f);
    S = std::fmaf(t2, S, 1.0f / 5.0f);
    S = std::fmaf(t2, S, 1.0f / 3.0f);
    S = std::fmaf(t2, S, 1.0f);
    S = S * t;
    const f32 lg = (g_lp_model & 2) ? std::fmaf(S, 2.885390081777927f, e - 127.0f)
                                    : (e - 127.0f) + S * 2.885390081777927f;
    const f32 y = std::max(p * lg, -126.0f);
    const f32 k = std::nearbyint(y);
    const f32 f = (y - k) * 0.6931471805599453f;
    f32 P = 1.0f / 720.0f;
    P = std::fmaf(f, P, 1.0f / 120.0f);
    P = std::fmaf(f, P, 1.0f / 24.0f);
    P = std::fmaf(f, P, 1.0f / 6.0f);
    P = std::fmaf(f, P, 0.5f);
    P = std::fmaf(f, P, 1.0f);
    P = std::fmaf(f, P, 1.0f);
    u32 pb;
    std::memcpy(&pb, &P, 4);
    pb += u32(int32_t(k)) << 23;
    f32 out;
    std::memcpy(&out, &pb, 4);
    return x < 1e-30f ? 0.0f : out;
}

f32 powf_ref(f32 x, f32 y) { return a64::ref_powf(x, y, (g_lp_model & 4) != 0); }

// kern::lp (metric.hpp:183-207).
f32 lp(const f32* a, const f32* b, u32 dim, f32 p) {
    const f32 M = linf(a, b, dim);
    if (M == 0.0f) return 0.0f;
    const f32 inv = 1.0f / M;
    const bool integral = p == std::floor(p) && p <= 8.0f;
    u32 k = 0;
    f32 s = 0.0f;
    if (!integral && dim >= 8) {
        f32 acc[8] = {0};
        for (; k + 8 <= dim; k += 8)
            for (int l = 0; l < 8; ++l)
                acc[l] = acc[l] + pow01(std::min(std::fabs(a[k + l] - b[k + l]) * inv, 1.0f), p);
        s = hsum8(acc);
    }
    for (; k < dim; ++k) {
        const f32 x = std::min(1.0f, std::fabs(a[k] - b[k]) * inv);
        s += integral ? ipow(x, u32(p)) : powf_ref(x, p);
    }
    return M * powf_ref(s, 1.0f / p);
}

f32 dist(int kind, f32 p, const f32* a, const f32* b, u32 dim) {
    switch (kind) {
        case 0: return l1(a, b, dim);
        case 1: return l2(a, b, dim);
        case 2: return linf(a, b, dim);
        default: return lp(a, b, dim, p);
    }
}

// ---------------------------------------------------------------------------
// Combinatorial number system (rips.hpp:72-93, :509-580).
// ---------------------------------------------------------------------------
u64 binom(u64 v, u32 k) {
    if (k > v) return 0;
    unsigned __int128 r = 1;
    for (u32 i = 0; i < k; ++i) r = r * (v - i) / (i + 1);
    return u64(r);
}

// Vertices (descending) of the simplex with nv vertices and index idx.
void decode(u64 idx, u32 nv, u32 n, u32* vd) {
    u32 top = n;
    for (u32 i = 0; i < nv; ++i) {
        const u32 k = nv - i;
        u32 lo = k - 1, hi = top;   // C(lo, k) <= idx < C(hi, k)
        while (hi - lo > 1) {
            const u32 mid = lo + (hi - lo) / 2;
            if (binom(mid, k) <= idx) lo = mid;
            else hi = mid;
        }
        vd[i] = lo;
        idx -= binom(lo, k);
        top = lo;
    }
}

u64 encode(const u32* vd, u32 nv) {   // vertices descending
    u64 s = 0;
    for (u32 i = 0; i < nv; ++i) s += binom(vd[i], nv - i);
    return s;
}

// ---------------------------------------------------------------------------
// A complex: dense full matrix or CSR (rips.hpp:262-472).
// ---------------------------------------------------------------------------
struct Cx {
    const f32* mat = nullptr;
    const u64* rp = nullptr;
    const u32* ci = nullptr;
    const f32* w = nullptr;
    u32 n = 0;
    f32 thr = INFINITY;

    f32 d(u32 i, u32 j) const {
        if (i == j) return 0.0f;
        if (mat) return mat[u64(i) * n + j];
        const u32* b = ci + rp[i];
        const u32* e = ci + rp[i + 1];
        const u32* it = std::lower_bound(b, e, j);
        return (it != e && *it == j) ? w[it - ci] : INFINITY;
    }

    // Cofacet candidates of vd (nv vertices, descending, diameter diam) in
    // DESCENDING order of the added vertex w, restricted to w > vd[0] unless
    // all; fn(w, t, cd) with t = #{vd > w} and cd the cofacet diameter, only
    // for cd <= cap. fn returns false to stop.
    template <typename F>
    void cofacets(const u32* vd, u32 nv, f32 diam, bool all, f32 cap, F&& fn) const {
        if (!mat) {
            // SparseComplex::cofacets (rips.hpp:429-471): the common
            // neighbours of vd's vertices, walked down from the top of their
            // sorted rows.
            u64 p[40], lo[40];
            for (u32 i = 0; i < nv; ++i) {
                lo[i] = rp[vd[i]];
                p[i] = rp[vd[i] + 1];
                if (p[i] == lo[i]) return;
            }
            for (;;) {
                u32 x = ci[p[0] - 1];
                bool agree = true;
                for (u32 i = 1; i < nv && agree; ++i) {
                    while (ci[p[i] - 1] > x) {
                        if (--p[i] == lo[i]) return;
                    }
                    if (ci[p[i] - 1] < x) {
                        x = ci[p[i] - 1];
                        agree = false;
                    }
                }
                if (!agree) {
                    while (ci[p[0] - 1] > x) {
                        if (--p[0] == lo[0]) return;
                    }
                    continue;
                }
                u32 t = 0;
                for (u32 i = 0; i < nv; ++i) t += vd[i] > x;
                if (!all && t > 0) return;
                f32 cd = diam;
                for (u32 i = 0; i < nv; ++i) cd = std::max(cd, w[p[i] - 1]);
                if (cd <= cap && !fn(x, t, cd)) return;
                if (--p[0] == lo[0]) return;
            }
        }
        for (int64_t wi = int64_t(n) - 1; wi >= 0; --wi) {
            const u32 w = u32(wi);
            u32 t = 0;
            bool in = false;
            for (u32 i = 0; i < nv; ++i) {
                if (vd[i] > w) ++t;
                if (vd[i] == w) in = true;
            }
            if (!all && t > 0) return;
            if (in) continue;
            f32 cd = diam;
            bool ok = true;
            for (u32 i = 0; i < nv && ok; ++i) {
                const f32 dv = d(vd[i], w);
                if (!(dv <= cap)) ok = false;   // absent edges are +inf
                cd = std::max(cd, dv);
            }
            if (ok && cd <= cap && !fn(w, t, cd)) return;
        }
    }

    // zero_pivot_cofacet_v (rips.hpp:585-605).
    u64 zero_cofacet(const u32* vd, u32 nv, f32 d, u32* cv) const {
        u64 found = kNone;
        cofacets(vd, nv, d, true, d, [&](u32 w, u32 t, f32) {
            for (u32 i = 0; i < t; ++i) cv[i] = vd[i];
            cv[t] = w;
            for (u32 i = t; i < nv; ++i) cv[i + 1] = vd[i];
            found = encode(cv, nv + 1);
            return false;
        });
        return found;
    }

    // zero_pivot_facet_v (rips.hpp:609-636): first facet in ascending index
    // order (vertex j = 0, 1, ... removed) with diameter d.
    u64 zero_facet(const u32* vd, u32 nv, f32 d, u32* fv) const {
        if (nv < 2) return kNone;
        for (u32 j = 0; j < nv; ++j) {
            bool hit = false;
            for (u32 a = 0; a < nv && !hit; ++a)
                for (u32 b = a + 1; b < nv && !hit; ++b)
                    hit = a != j && b != j && this->d(vd[a], vd[b]) == d;
            if (hit) {
                for (u32 i = 0, o = 0; i < nv; ++i)
                    if (i != j) fv[o++] = vd[i];
                return encode(fv, nv - 1);
            }
        }
        return kNone;
    }

    // zero_apparent_cofacet_v / zero_apparent_facet_v (rips.hpp:638-649).
    bool apparent_cofacet(const u32* vd, u32 nv, u64 idx, f32 d) const {
        u32 cv[40], fv[40];
        const u64 c = zero_cofacet(vd, nv, d, cv);
        return c != kNone && zero_facet(cv, nv + 1, d, fv) == idx;
    }
    bool apparent_facet(const u32* vd, u32 nv, u64 idx, f32 d) const {
        u32 cv[40], fv[40];
        const u64 f = zero_facet(vd, nv, d, fv);
        return f != kNone && zero_cofacet(fv, nv - 1, d, cv) == idx;
    }
};

// precedes (rips.hpp:114-118): (d ascending, index descending).
struct E {
    u64 idx;
    f32 d;
};
bool precedes(const E& a, const E& b) { return a.d < b.d || (a.d == b.d && a.idx > b.idx); }

std::vector<E> kept_edges(const Cx& cx) {
    std::vector<E> e;
    for (u32 i = 1; i < cx.n; ++i) {
        if (cx.mat) {
            for (u32 j = 0; j < i; ++j) {
                const f32 d = cx.mat[u64(i) * cx.n + j];
                if (d <= cx.thr) e.push_back({u64(i) * (i - 1) / 2 + j, d});
            }
        } else {
            for (u64 t = cx.rp[i]; t < cx.rp[i + 1]; ++t)
                if (cx.ci[t] < i && cx.w[t] <= cx.thr) e.push_back({u64(i) * (i - 1) / 2 + cx.ci[t], cx.w[t]});
        }
    }
    return e;
}

struct UF {
    std::vector<u32> p, r;
    explicit UF(u32 n) : p(n), r(n, 0) { std::iota(p.begin(), p.end(), 0u); }
    u32 find(u32 x) {
        while (p[x] != x) x = p[x] = p[p[x]];
        return x;
    }
    bool unite(u32 a, u32 b) {
        a = find(a);
        b = find(b);
        if (a == b) return false;
        if (r[a] < r[b]) std::swap(a, b);
        p[b] = a;
        if (r[a] == r[b]) ++r[a];
        return true;
    }
};

std::vector<std::vector<std::pair<u32, f32>>> rows_from_lists(const f32* x, u32 n, u32 dim, int kind,
                                                              f32 p, const u32* ids, u32 k) {
    std::vector<std::vector<std::pair<u32, f32>>> rows(n);
    for (u32 i = 0; i < n; ++i)
        for (u32 t = 0; t < k; ++t) {
            const u32 j = ids[u64(i) * k + t];
            if (j == i) continue;
            rows[i].emplace_back(j, 0.0f);
            rows[j].emplace_back(i, 0.0f);
        }
    for (u32 v = 0; v < n; ++v) {
        auto& r = rows[v];
        std::sort(r.begin(), r.end());
        r.erase(std::unique(r.begin(), r.end(), [](auto& a, auto& b) { return a.first == b.first; }), r.end());
        for (auto& e : r) e.second = dist(kind, p, x + u64(v) * dim, x + u64(e.first) * dim, dim);
    }
    return rows;
}

}  // namespace

extern "C" {

void or_set_lp_model(int model) { g_lp_model = model; }
int or_get_lp_model(void) { return g_lp_model; }
float or_powf(float x, float y) { return powf_ref(x, y); }
float or_rcp(float x) { return a64::rcp_ps(x); }

float or_dist(int kind, float p, const float* a, const float* b, uint32_t dim) {
    return dist(kind, p, a, b, dim);
}

void or_dense(const float* x, uint32_t n, uint32_t dim, int kind, float p, float* mat) {
    for (u64 i = 0; i < n; ++i) {
        mat[i * n + i] = 0.0f;
        for (u32 j = 0; j < i; ++j) mat[i * n + j] = dist(kind, p, x + i * dim, x + u64(j) * dim, dim);
    }
    for (u64 i = 0; i < n; ++i)
        for (u32 j = u32(i) + 1; j < n; ++j) mat[i * n + j] = mat[u64(j) * n + i];
}

float or_enclosing_radius(const float* mat, uint32_t n) {
    f32 best = INFINITY;
    for (u64 i = 0; i < n; ++i) {
        f32 m = 0.0f;
        for (u32 j = 0; j < n; ++j) m = std::max(m, i == j ? 0.0f : mat[i * n + j]);
        best = std::min(best, m);
    }
    return best;
}

uint64_t or_dim0(const float* mat, const uint64_t* rp, const uint32_t* ci, const float* w,
                 uint32_t n, float thr, uint32_t maxdim, uint64_t* eidx, float* ed, uint8_t* app,
                 uint64_t* cidx, float* cd, uint64_t* ncols, float* h0, uint64_t* nh0) {
    Cx cx{mat, rp, ci, w, n, thr};
    std::vector<E> edges = kept_edges(cx);
    std::sort(edges.begin(), edges.end(), precedes);
    UF uf(n);
    std::vector<E> cols;
    u64 nb = 0;
    for (u64 i = 0; i < edges.size(); ++i) {
        const E e = edges[i];
        u32 vd[2];
        decode(e.idx, 2, n, vd);
        const bool a = maxdim >= 1 && cx.apparent_cofacet(vd, 2, e.idx, e.d);
        eidx[i] = e.idx;
        ed[i] = e.d;
        app[i] = a;
        if (uf.unite(vd[0], vd[1])) {
            if (e.d > 0.0f) { h0[2 * nb] = 0.0f; h0[2 * nb + 1] = e.d; ++nb; }
        } else if (maxdim >= 1 && !a) {
            cols.push_back(e);
        }
    }
    for (u32 v = 0; v < n; ++v)
        if (uf.find(v) == v) { h0[2 * nb] = 0.0f; h0[2 * nb + 1] = INFINITY; ++nb; }
    std::reverse(cols.begin(), cols.end());
    for (u64 i = 0; i < cols.size(); ++i) { cidx[i] = cols[i].idx; cd[i] = cols[i].d; }
    *ncols = cols.size();
    *nh0 = nb;
    return edges.size();
}

void or_emergent(const float* mat, const uint64_t* rp, const uint32_t* ci, const float* w,
                 uint32_t n, const uint64_t* cidx, const float* cd, uint64_t ncols,
                 uint64_t* cf_idx, float* cf_d, uint8_t* cf_app) {
    Cx cx{mat, rp, ci, w, n, INFINITY};
    for (u64 c = 0; c < ncols; ++c) {
        u32 vd[2], cv[3];
        decode(cidx[c], 2, n, vd);
        const u64 f = cx.zero_cofacet(vd, 2, cd[c], cv);
        cf_idx[c] = f;
        cf_d[c] = f == kNone ? 0.0f : cd[c];
        cf_app[c] = f != kNone && cx.apparent_facet(cv, 3, f, cd[c]);
    }
}

uint64_t or_assemble(const float* mat, uint32_t n, float thr, const uint64_t* sidx, const float* sd,
                     uint64_t ns, const uint64_t* piv, uint64_t npiv, uint64_t* cidx, float* cd,
                     uint64_t cap, uint64_t* napp) {
    Cx cx{mat, nullptr, nullptr, nullptr, n, thr};
    std::vector<E> cols;
    u64 skipped = 0;
    for (u64 s = 0; s < ns; ++s) {
        u32 vd[2];
        decode(sidx[s], 2, n, vd);
        cx.cofacets(vd, 2, sd[s], false, thr, [&](u32 wv, u32 t, f32 c) {
            u32 cv[3];
            for (u32 i = 0; i < t; ++i) cv[i] = vd[i];
            cv[t] = wv;
            for (u32 i = t; i < 2; ++i) cv[i + 1] = vd[i];
            const u64 idx = encode(cv, 3);
            if (std::binary_search(piv, piv + npiv, idx)) return true;
            if (cx.apparent_cofacet(cv, 3, idx, c) || cx.apparent_facet(cv, 3, idx, c)) {
                ++skipped;
                return true;
            }
            cols.push_back({idx, c});
            return true;
        });
    }
    std::sort(cols.begin(), cols.end(), [](const E& a, const E& b) { return precedes(b, a); });
    for (u64 i = 0; i < cols.size() && i < cap; ++i) { cidx[i] = cols[i].idx; cd[i] = cols[i].d; }
    *napp = skipped;
    return cols.size();
}

void or_knn(const float* x, uint32_t n, uint32_t dim, int kind, float p, uint32_t k, uint32_t* ids) {
    or_knn_rows(x, n, dim, kind, p, k, 0, n, 1, ids);
}

// Rows [q0, q1) of the kNN lists (ids holds rows q0.. at stride k), on
// `threads` host threads; the CPU-baseline leg of the benchmark times this.
void or_knn_rows(const float* x, uint32_t n, uint32_t dim, int kind, float p, uint32_t k, uint32_t q0,
                 uint32_t q1, uint32_t threads, uint32_t* ids) {
    k = n ? std::min<u32>(k, n - 1) : 0;
    // knn_query's bounded max-heap of (distance, id) (graph.hpp:123-166),
    // over every candidate instead of the k-d tree's leaves.
    auto work = [&](u32 lo, u32 hi) {
        std::vector<std::pair<f32, u32>> h;
        for (u32 i = lo; i < hi; ++i) {
            h.clear();
            for (u32 j = 0; j < n; ++j) {
                if (j == i) continue;
                const std::pair<f32, u32> c{dist(kind, p, x + u64(i) * dim, x + u64(j) * dim, dim), j};
                if (h.size() < k) {
                    h.push_back(c);
                    std::push_heap(h.begin(), h.end());
                } else if (c < h.front()) {
                    std::pop_heap(h.begin(), h.end());
                    h.back() = c;
                    std::push_heap(h.begin(), h.end());
                }
            }
            std::sort(h.begin(), h.end());
            for (u32 t = 0; t < k; ++t) ids[u64(i - q0) * k + t] = h[t].second;
        }
    };
    threads = std::max<u32>(1, std::min<u32>(threads, q1 > q0 ? q1 - q0 : 1));
    std::vector<std::thread> pool;
    for (u32 t = 0; t < threads; ++t) {
        const u32 lo = q0 + u32(u64(q1 - q0) * t / threads), hi = q0 + u32(u64(q1 - q0) * (t + 1) / threads);
        pool.emplace_back(work, lo, hi);
    }
    for (auto& th : pool) th.join();
}

uint64_t or_knn_graph(const float* x, uint32_t n, uint32_t dim, int kind, float p,
                      const uint32_t* ids, uint32_t k, uint64_t* rp, uint32_t* ci, float* w) {
    auto rows = rows_from_lists(x, n, dim, kind, p, ids, k);
    rp[0] = 0;
    for (u32 v = 0; v < n; ++v) {
        rp[v + 1] = rp[v] + rows[v].size();
        for (u64 t = 0; t < rows[v].size(); ++t) { ci[rp[v] + t] = rows[v][t].first; w[rp[v] + t] = rows[v][t].second; }
    }
    return rp[n];
}

uint64_t or_radius_graph(const float* x, uint32_t n, uint32_t dim, int kind, float p, float tau,
                         uint64_t* rp, uint32_t* ci, float* w, uint64_t cap) {
    u64 o = 0;
    rp[0] = 0;
    for (u32 i = 0; i < n; ++i) {
        for (u32 j = 0; j < n; ++j) {
            if (j == i) continue;
            const f32 d = dist(kind, p, x + u64(i) * dim, x + u64(j) * dim, dim);
            if (d <= tau) {
                if (o < cap) { ci[o] = j; w[o] = d; }
                ++o;
            }
        }
        rp[i + 1] = o;
    }
    return o;
}

uint64_t or_mst_h0(const float* x, uint32_t n, uint32_t dim, int kind, float p, float thr, float* bars) {
    if (n == 0) return 0;
    std::vector<f32> best(n, INFINITY), deaths;
    std::vector<u8> in(n, 0);
    u32 cur = 0;
    in[0] = 1;
    for (u32 step = 1; step < n; ++step) {
        f32 bd = INFINITY;
        u32 bj = ~0u;
        for (u32 j = 0; j < n; ++j) {
            if (in[j]) continue;
            best[j] = std::min(best[j], dist(kind, p, x + u64(cur) * dim, x + u64(j) * dim, dim));
            if (best[j] < bd || (best[j] == bd && j < bj)) { bd = best[j]; bj = j; }
        }
        deaths.push_back(bd);
        in[bj] = 1;
        cur = bj;
    }
    std::sort(deaths.begin(), deaths.end());
    u64 nb = 0, essential = 1;
    for (f32 d : deaths) {
        if (d > thr) ++essential;
        else if (d > 0.0f) { bars[2 * nb] = 0.0f; bars[2 * nb + 1] = d; ++nb; }
    }
    for (u64 e = 0; e < essential; ++e) { bars[2 * nb] = 0.0f; bars[2 * nb + 1] = INFINITY; ++nb; }
    return nb;
}

uint64_t or_redzed_edges(const float* mat, const uint64_t* rp, const uint32_t* ci, const float* w,
                         uint32_t n, float thr, float* d, int32_t* verts) {
    Cx cx{mat, rp, ci, w, n, thr};
    std::vector<E> e = kept_edges(cx);
    std::sort(e.begin(), e.end(), [](const E& a, const E& b) { return a.d < b.d || (a.d == b.d && a.idx < b.idx); });
    for (u64 i = 0; i < e.size(); ++i) {
        u32 vd[2];
        decode(e[i].idx, 2, n, vd);
        d[i] = e[i].d;
        verts[2 * i] = int32_t(vd[1]);
        verts[2 * i + 1] = int32_t(vd[0]);
    }
    return e.size();
}

}  // extern "C"
