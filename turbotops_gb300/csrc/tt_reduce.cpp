// tt_reduce.cpp — host cohomology reduction of the columns the GPU front end
// leaves (rips.hpp Reducer::compute_pairs, :874-978: the reduction stays
// sequential on the host by design).
//
// The algorithm is Ripser's (U. Bauer, J. Appl. Comput. Topol. 2021) as the
// reference runs it: columns in descending filtration order (d desc, index
// asc); each column's coboundary in a priority queue ordered by (d asc, index
// desc) with mod-2 cancellation at the top; a pivot already owned by an
// earlier column adds that column's stored reduction; a pivot with a
// zero-apparent facet adds that facet's coboundary; otherwise the pivot pairs
// the column (a bar if it is longer than zero). The emergent-pair shortcut
// (:903-928) pairs a column with its first zero cofacet when no earlier
// column owns it and it has no zero-apparent facet; for dimension 1 the GPU
// supplies that cofacet and flag per column, and only the ownership lookup
// runs here.
//
// Only the priority queue differs from the reference's binary heap: diameter
// buckets read as sorted runs (BucketQueue), 64-bit packed keys where every
// index of the dimension fits in 32 bits, and, on dense complexes, a push
// frontier that leaves the cofacets beyond the column's current reach owed
// instead of queued. Equal entries are indistinguishable and surface in the
// same order, so the pivots, the stored reductions and the pairs are the
// reference's.
#include "tt_reduce.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <limits>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>

namespace tt {
namespace host {

namespace {

#ifndef TT_FRONT
#define TT_FRONT 8
#endif

constexpr uint64_t kNone = std::numeric_limits<uint64_t>::max();

inline bool precedes(const Entry& a, const Entry& b) { return a.d < b.d || (a.d == b.d && a.idx > b.idx); }

// Order-preserving bits of a diameter (>= 0 or +inf; -0 is taken as +0,
// which it equals) and back.
inline uint32_t dbits(float d) {
    uint32_t u;
    std::memcpy(&u, &d, 4);
    u = u == 0x80000000u ? 0u : u;
    return u ^ ((0u - (u >> 31)) | 0x80000000u);   // negative: ~u; else u | sign bit
}
inline float from_dbits(uint32_t u) {
    u = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    float d;
    std::memcpy(&d, &u, 4);
    return d;
}

// C(v, k) for v <= n, k <= K, overflow-checked.
struct Binom {
    uint32_t n = 0, K = 0;
    std::vector<uint64_t> t;   // t[k * (n + 1) + v]
    Binom(uint32_t nn, uint32_t KK) : n(nn), K(KK), t(uint64_t(nn + 1) * (KK + 1), 0) {
        for (uint32_t v = 0; v <= n; ++v) {
            at(v, 0) = 1;
            for (uint32_t k = 1; k <= std::min(v, K); ++k) {
                uint64_t s;
                if (__builtin_add_overflow(at(v - 1, k - 1), at(v - 1, k), &s))
                    throw std::overflow_error("rips: simplex index overflow");
                at(v, k) = s;
            }
        }
    }
    uint64_t& at(uint32_t v, uint32_t k) { return t[uint64_t(k) * (n + 1) + v]; }
    uint64_t operator()(uint32_t v, uint32_t k) const { return k > K ? 0 : t[uint64_t(k) * (n + 1) + v]; }
    const uint64_t* row(uint32_t k) const { return t.data() + uint64_t(k) * (n + 1); }   // k <= K
};

struct Cx {
    const HostComplex& c;
    const Binom& B;
    mutable std::vector<float> cdw;      // dense: diameter of the cofacet through each vertex
    mutable std::vector<uint32_t> ubw;   // and its order-preserving bits

    float dist(uint32_t i, uint32_t j) const {
        if (i == j) return 0.0f;
        if (c.mat) return c.mat[uint64_t(i) * c.n + j];
        const uint32_t* b = c.ci + c.rp[i];
        const uint32_t* e = c.ci + c.rp[i + 1];
        const uint32_t* it = std::lower_bound(b, e, j);
        return (it != e && *it == j) ? c.w[it - c.ci] : INFINITY;
    }

    // vertices of the simplex with nv vertices, descending (rips.hpp decode)
    void decode(uint64_t idx, uint32_t nv, uint32_t* vd) const {
        uint32_t top = c.n;
        for (uint32_t i = 0; i < nv; ++i) {
            const uint32_t k = nv - i;
            uint32_t lo = k - 1, hi = top;
            while (hi - lo > 1) {
                const uint32_t mid = lo + (hi - lo) / 2;
                if (B(mid, k) <= idx) lo = mid;
                else hi = mid;
            }
            vd[i] = lo;
            idx -= B(lo, k);
            top = lo;
        }
    }

    // Cofacets of vd (nv vertices, descending, diameter diam) with diameter
    // <= cap, in descending index order: fn(Entry, w, t) -> continue?
    template <typename F>
    void cofacets(const uint32_t* vd, uint32_t nv, float diam, float cap, F&& fn) const {
        uint64_t A[34], S[34];
        A[0] = 0;
        for (uint32_t i = 0; i < nv; ++i) A[i + 1] = A[i] + B(vd[i], nv + 1 - i);
        S[nv] = 0;
        for (uint32_t i = nv; i-- > 0;) S[i] = S[i + 1] + B(vd[i], nv - i);
        if (c.mat) {
            uint32_t t = 0;
            for (int64_t wi = int64_t(c.n) - 1; wi >= 0; --wi) {
                const uint32_t w = uint32_t(wi);
                while (t < nv && vd[t] > w) ++t;
                if (t < nv && vd[t] == w) continue;
                float cd = diam;
                bool ok = true;
                for (uint32_t i = 0; i < nv; ++i) {
                    const float dv = c.mat[uint64_t(vd[i]) * c.n + w];
                    if (dv > cd) {
                        cd = dv;
                        if (cd > cap) { ok = false; break; }
                    }
                }
                if (ok && !fn(Entry{A[t] + B(w, nv + 1 - t) + S[t], cd}, w, t)) return;
            }
            return;
        }
        // CSR: common neighbours walked down from the top of the sorted rows
        if (nv == 2) {   // an edge: two rows, the smaller head steps without a branch
            const uint32_t a = vd[0], b = vd[1];
            uint64_t pa = c.rp[a + 1], pb = c.rp[b + 1];
            const uint64_t la = c.rp[a], lb = c.rp[b];
            while (pa > la && pb > lb) {
                const uint32_t xa = c.ci[pa - 1], xb = c.ci[pb - 1];
                if (xa != xb) {
                    pa -= xa > xb;
                    pb -= xb > xa;
                    continue;
                }
                const uint32_t t = uint32_t(a > xa) + uint32_t(b > xa);
                const float cd = std::max(diam, std::max(c.w[pa - 1], c.w[pb - 1]));
                if (cd <= cap && !fn(Entry{A[t] + B(xa, 3 - t) + S[t], cd}, xa, t)) return;
                --pa;
                --pb;
            }
            return;
        }
        uint64_t p[34], lo[34];
        for (uint32_t i = 0; i < nv; ++i) {
            lo[i] = c.rp[vd[i]];
            p[i] = c.rp[vd[i] + 1];
            if (p[i] == lo[i]) return;
        }
        for (;;) {
            uint32_t x = c.ci[p[0] - 1];
            bool agree = true;
            for (uint32_t i = 1; i < nv && agree; ++i) {
                while (c.ci[p[i] - 1] > x)
                    if (--p[i] == lo[i]) return;
                if (c.ci[p[i] - 1] < x) {
                    x = c.ci[p[i] - 1];
                    agree = false;
                }
            }
            if (!agree) {
                while (c.ci[p[0] - 1] > x)
                    if (--p[0] == lo[0]) return;
                continue;
            }
            uint32_t t = 0;
            while (t < nv && vd[t] > x) ++t;
            float cd = diam;
            for (uint32_t i = 0; i < nv; ++i) cd = std::max(cd, c.w[p[i] - 1]);
            if (cd <= cap && !fn(Entry{A[t] + B(x, nv + 1 - t) + S[t], cd}, x, t)) return;
            if (--p[0] == lo[0]) return;
        }
    }

    // The cofacets with diameter <= cap whose diameter bits lie in (lo, hi],
    // in the order of cofacets(): fn(Entry). Returns the smallest diameter
    // bits above hi among the cofacets with diameter <= cap (UINT32_MAX when
    // there is none). Dense: the diameters through all vertices are taken row
    // by row first, then emitted per range of vertices between the simplex's
    // own, where the index is one binomial row plus a constant.
    template <typename F>
    uint32_t window_cofacets(const uint32_t* vd, uint32_t nv, float diam, float cap, uint32_t lo, uint32_t hi,
                             F&& fn) const {
        const uint32_t cb = dbits(cap);
        hi = std::min(hi, cb);
        uint32_t above = UINT32_MAX;
        if (!c.mat) {
            cofacets(vd, nv, diam, cap, [&](const Entry& e, uint32_t, uint32_t) {
                const uint32_t u = dbits(e.d);
                if (u > hi) above = std::min(above, u);
                else if (u > lo) fn(e);
                return true;
            });
            return above;
        }
        const uint32_t n = c.n;
        cdw.resize(n);
        ubw.resize(n);
        float* cd = cdw.data();
        uint32_t* ub = ubw.data();
        const float* r0 = c.mat + uint64_t(vd[0]) * n;
        for (uint32_t w = 0; w < n; ++w) cd[w] = std::max(diam, r0[w]);
        for (uint32_t i = 1; i < nv; ++i) {
            const float* r = c.mat + uint64_t(vd[i]) * n;
            for (uint32_t w = 0; w < n; ++w) cd[w] = std::max(cd[w], r[w]);
        }
        // diameter bits, the simplex's own vertices outside every window
        for (uint32_t w = 0; w < n; ++w) ub[w] = dbits(cd[w]);
        for (uint32_t i = 0; i < nv; ++i) ub[vd[i]] = UINT32_MAX;
        for (uint32_t w = 0; w < n; ++w) {
            const uint32_t owed = uint32_t(ub[w] > hi) & uint32_t(ub[w] <= cb);
            above = std::min(above, ub[w] | (owed - 1u));   // not owed: UINT32_MAX
        }
        if (hi <= lo) return above;
        const uint32_t width = hi - lo;   // u in (lo, hi]: u - lo - 1 < width
        uint64_t A = 0, S[34];
        S[nv] = 0;
        for (uint32_t i = nv; i-- > 0;) S[i] = S[i + 1] + B(vd[i], nv - i);
        uint32_t top = n;   // w in [bot, top): the vertices above vd[t] and below vd[t - 1]
        for (uint32_t t = 0; t <= nv; ++t) {
            const uint32_t bot = t < nv ? vd[t] + 1 : 0;
            const uint64_t base = A + S[t];
            const uint64_t* Bk = B.row(nv + 1 - t);
            for (uint32_t w = top; w-- > bot;)
                if (ub[w] - lo - 1 < width) fn(Entry{base + Bk[w], cd[w]});
            if (t < nv) {
                A += B(vd[t], nv + 1 - t);
                top = vd[t];
            }
        }
        return above;
    }

    // first cofacet in descending order with diameter d (its vertices in cv)
    uint64_t zero_cofacet(const uint32_t* vd, uint32_t nv, float d, uint32_t* cv) const {
        uint64_t found = kNone;
        cofacets(vd, nv, d, d, [&](const Entry& e, uint32_t w, uint32_t t) {
            found = e.idx;
            for (uint32_t i = 0; i < t; ++i) cv[i] = vd[i];
            cv[t] = w;
            for (uint32_t i = t; i < nv; ++i) cv[i + 1] = vd[i];
            return false;
        });
        return found;
    }

    // first facet in ascending order with diameter d (its vertices in fv)
    uint64_t zero_facet(const uint32_t* vd, uint32_t nv, float d, uint32_t* fv) const {
        if (nv < 2) return kNone;
        float dm[33][33];
        for (uint32_t a = 0; a < nv; ++a)
            for (uint32_t b = a + 1; b < nv; ++b) dm[a][b] = dist(vd[a], vd[b]);
        for (uint32_t j = 0; j < nv; ++j) {
            bool hit = false;
            for (uint32_t a = 0; a < nv && !hit; ++a)
                for (uint32_t b = a + 1; b < nv && !hit; ++b) hit = a != j && b != j && dm[a][b] == d;
            if (hit) {
                uint64_t idx = 0;
                for (uint32_t i = 0, o = 0; i < nv; ++i)
                    if (i != j) {
                        fv[o] = vd[i];
                        idx += B(vd[i], nv - 1 - o);
                        ++o;
                    }
                return idx;
            }
        }
        return kNone;
    }

    // zero_apparent_cofacet_v / zero_apparent_facet_v (rips.hpp:637-648) of
    // the simplex s with vertices vd (nv, descending): is s in a zero-apparent
    // pair, as the cofacet's facet or as the facet's cofacet?
    bool in_zero_apparent_pair(const uint32_t* vd, uint32_t nv, const Entry& s) const {
        uint32_t cv[34], fv[34], gv[34];
        const uint64_t c = zero_cofacet(vd, nv, s.d, cv);
        if (c != kNone && zero_facet(cv, nv + 1, s.d, gv) == s.idx) return true;
        const uint64_t f = zero_facet(vd, nv, s.d, fv);
        return f != kNone && zero_cofacet(fv, nv - 1, s.d, gv) == s.idx;
    }

    // zero_apparent_facet: the zero facet whose zero cofacet is s
    Entry zero_apparent_facet(const Entry& s, uint32_t nv) const {
        uint32_t vd[34], fv[34], cv[34];
        decode(s.idx, nv, vd);
        const uint64_t f = zero_facet(vd, nv, s.d, fv);
        if (f == kNone) return Entry{kNone, 0};
        return zero_cofacet(fv, nv - 1, s.d, cv) == s.idx ? Entry{f, s.d} : Entry{kNone, 0};
    }
};

// Open-addressing map: simplex index -> column.
struct PivotMap {
    std::vector<uint64_t> k, v;
    uint64_t mask = 0, count = 0;
    explicit PivotMap(uint64_t cap) {
        uint64_t c = 16;
        while (c < 2 * cap + 2) c <<= 1;
        k.assign(c, kNone);
        v.assign(c, 0);
        mask = c - 1;
    }
    static uint64_t h(uint64_t x) {
        x ^= x >> 33;
        x *= 0xff51afd7ed558ccdull;
        x ^= x >> 33;
        return x;
    }
    uint64_t find(uint64_t key) const {
        for (uint64_t s = h(key) & mask;; s = (s + 1) & mask) {
            if (k[s] == key) return v[s];
            if (k[s] == kNone) return kNone;
        }
    }
    void insert(uint64_t key, uint64_t val) {
        if (2 * (count + 1) > k.size()) grow();
        uint64_t s = h(key) & mask;
        while (k[s] != kNone && k[s] != key) s = (s + 1) & mask;
        if (k[s] == kNone) ++count;
        k[s] = key;
        v[s] = val;
    }
    void grow() {
        std::vector<uint64_t> ok, ov;
        ok.swap(k);
        ov.swap(v);
        k.assign(ok.size() * 2, kNone);
        v.assign(ok.size() * 2, 0);
        mask = k.size() - 1;
        count = 0;
        for (uint64_t i = 0; i < ok.size(); ++i)
            if (ok[i] != kNone) insert(ok[i], ov[i]);
    }
};

// What the working coboundary stores per entry: the Entry itself, or, when
// every index of the dimension fits in 32 bits, one 64-bit key (diameter
// bits above the complemented index) whose integer order is the filtration
// order — half the bytes, and compares without branches.
struct WideKey {
    using T = Entry;
    static T make(const Entry& e) { return e; }
    static Entry entry(const T& t) { return t; }
    static bool less(const T& a, const T& b) { return precedes(a, b); }
    static bool same(const T& a, const T& b) { return a.idx == b.idx; }
    static uint32_t bits(const T& t) { return dbits(t.d); }
};
struct PackedKey {
    using T = uint64_t;
    static T make(const Entry& e) { return uint64_t(dbits(e.d)) << 32 | (0xffffffffu - uint32_t(e.idx)); }
    static Entry entry(T t) { return Entry{0xffffffffu - uint32_t(t), from_dbits(uint32_t(t >> 32))}; }
    static bool less(T a, T b) { return a < b; }
    static bool same(T a, T b) { return a == b; }
    static uint32_t bits(T t) { return uint32_t(t >> 32); }
};

// The working coboundary: a priority queue in filtration order (smallest
// diameter first, larger index first among equal diameters) with pairwise
// cancellation of equal indices at the top. Entries go into buckets by their
// diameter bits between the column's birth (no entry is earlier) and the
// largest diameter of the complex. A push is an append to one of few enough
// buckets that their tails stay in cache: most entries of a column lie
// beyond its pivot and are never looked at again. The lowest non-empty
// bucket is sorted when it comes to the top and read with a cursor. Entries
// pushed into it after that are sorted at the next read and merged into a
// second, smaller sorted run (folded into the first when it grows past an
// eighth of it); the front is the earlier of the two runs' heads. Buckets
// are monotone in the diameter and equal keys share a bucket, so the entries
// surface in exactly the order of a single heap over the whole column.
template <class K>
struct BucketQueue {
    using T = typename K::T;
    static constexpr uint32_t kBits = 10, kBuckets = 1u << kBits;
    std::vector<std::vector<T>> bk = std::vector<std::vector<T>>(kBuckets);
    std::vector<uint64_t> live = std::vector<uint64_t>(kBuckets / 64, 0);   // non-empty buckets
    std::vector<T> aux, pend, tmp;   // second run, pushes since the last read, merge buffer
    uint32_t cur = kBuckets;         // buckets below cur are empty
    bool ready = false;              // bk[cur] is sorted from pos on, aux from apos on
    size_t pos = 0, apos = 0;
    uint32_t lo = 0, shift = 0;
    uint64_t count = 0;

    // Empties the queue; entries of the next column are expected in [a, b]
    // (outside it they only share the end buckets).
    void reset(float a, float b) {
        for (uint32_t w = 0; w < kBuckets / 64; ++w) {
            for (uint64_t m = live[w]; m; m &= m - 1) bk[(w << 6) + uint32_t(__builtin_ctzll(m))].clear();
            live[w] = 0;
        }
        aux.clear();
        pend.clear();
        lo = dbits(a);
        const uint32_t span = dbits(b) > lo ? dbits(b) - lo : 0;
        shift = 0;
        while ((span >> shift) >= kBuckets) ++shift;
        cur = kBuckets;
        ready = false;
        pos = apos = 0;
        count = 0;
    }
    uint32_t bucket(uint32_t u) const {
        if (u <= lo) return 0;
        const uint32_t x = (u - lo) >> shift;
        return x < kBuckets ? x : kBuckets - 1;
    }
    void mark(uint32_t x) { live[x >> 6] |= 1ull << (x & 63); }
    void unmark(uint32_t x) { live[x >> 6] &= ~(1ull << (x & 63)); }
    // merges the unread parts of v (from *vp) and w (from wp) into v
    void merge_into(std::vector<T>& v, size_t* vp, const std::vector<T>& w, size_t wp) {
        tmp.resize(v.size() - *vp + w.size() - wp);
        std::merge(v.begin() + ptrdiff_t(*vp), v.end(), w.begin() + ptrdiff_t(wp), w.end(), tmp.begin(), K::less);
        v.swap(tmp);
        *vp = 0;
    }
    // turns the current bucket back into an unsorted one
    void unready() {
        std::vector<T>& v = bk[cur];
        v.erase(v.begin(), v.begin() + ptrdiff_t(pos));
        v.insert(v.end(), aux.begin() + ptrdiff_t(apos), aux.end());
        v.insert(v.end(), pend.begin(), pend.end());
        aux.clear();
        pend.clear();
        pos = apos = 0;
        ready = false;
        if (v.empty()) unmark(cur);
    }
    void push(const Entry& e) {
        const T t = K::make(e);
        const uint32_t x = bucket(K::bits(t));
        ++count;
        if (ready && x == cur) {
            pend.push_back(t);
            return;
        }
        if (ready && x < cur) unready();
        bk[x].push_back(t);
        mark(x);
        if (x < cur) cur = x;
    }
    // the lowest non-empty bucket sorted under the cursors (count > 0, so a
    // push has set cur below kBuckets)
    void settle() {
        if (ready) {
            if (!pend.empty()) {
                std::sort(pend.begin(), pend.end(), K::less);
                merge_into(aux, &apos, pend, 0);
                pend.clear();
                if (8 * aux.size() > bk[cur].size() - pos) {
                    merge_into(bk[cur], &pos, aux, 0);
                    aux.clear();
                }
            }
            if (pos < bk[cur].size() || apos < aux.size()) return;
            bk[cur].clear();
            aux.clear();
            unmark(cur);
            ready = false;
        }
        uint32_t w = cur >> 6;
        uint64_t m = live[w] & (~0ull << (cur & 63));
        while (!m) m = live[++w];
        cur = (w << 6) + uint32_t(__builtin_ctzll(m));
        std::sort(bk[cur].begin(), bk[cur].end(), K::less);
        pos = apos = 0;
        ready = true;
    }
    // The first entry that does not cancel, left in the queue (idx kNone when
    // everything cancels).
    Entry get_pivot() {
        T piv{};
        bool have = false, in_aux = false;
        while (count) {
            settle();
            const std::vector<T>& v = bk[cur];
            const bool fa = apos < aux.size() && (pos == v.size() || K::less(aux[apos], v[pos]));
            const T f = fa ? aux[apos] : v[pos];
            if (!have) {
                piv = f;
                have = true;
                in_aux = fa;
            } else if (K::same(f, piv)) {
                have = false;
            } else {
                break;
            }
            if (fa) ++apos;
            else ++pos;
            --count;
        }
        if (!have) return Entry{kNone, 0};
        // still in the run it was read from unless that bucket ran out
        size_t& p = in_aux ? apos : pos;
        const std::vector<T>& v = in_aux ? aux : bk[cur];
        if (ready && p > 0 && p <= v.size() && K::same(v[p - 1], piv)) {
            --p;
            ++count;
            return K::entry(piv);
        }
        const Entry e = K::entry(piv);
        push(e);
        return e;
    }
};

}  // namespace

namespace {

// One column's reduction with its own working state (so that several run at
// once): cols[c] is reduced, as compute_pairs does, until its pivot has no
// owner in `pivots` and no zero-apparent facet (or the column cancels out),
// reading the stored reductions (off / red) of the owners it meets. The
// simplices it added are left in wr.
template <class K>
struct ColumnReducer {
    const HostComplex& hc;
    const Cx cx;
    const uint32_t nv;
    float dmax = 0;
    uint32_t top_bits = 0;
    BucketQueue<K> wc;
    std::vector<Entry> owed, owed2, wr;
    uint32_t vd[34];
    uint32_t front = 0, grow = 1, owed_min = UINT32_MAX;

    ColumnReducer(const HostComplex& h, const Binom& B, uint32_t dim, float dm)
        : hc(h), cx{h, B, {}, {}}, nv(dim + 1), dmax(dm), top_bits(dbits(dm)) {}

    // Push frontier (dense complexes). Only cofacets whose diameter bits are
    // at most `front` go into the queue; a simplex with cofacets above it is
    // owed them, and owed_min is the smallest owed diameter. The queue's first
    // entry that does not cancel is then the column's pivot, since every owed
    // entry comes later in the filtration order; when the queue cancels out,
    // the frontier moves past owed_min (by a width that doubles each time) and
    // the owed simplices push their cofacets in the new window. Most cofacets
    // of a column lie far beyond its pivot and are never pushed at all.
    void push_window(const Entry& s, uint32_t lo, std::vector<Entry>& still) {
        cx.decode(s.idx, nv, vd);
        const uint32_t a = cx.window_cofacets(vd, nv, s.d, hc.thr, lo, front, [&](const Entry& e) { wc.push(e); });
        if (a != UINT32_MAX) {
            still.push_back(s);
            owed_min = std::min(owed_min, a);
        }
    }
    void push_coboundary(const Entry& s) { push_window(s, 0, owed); }
    Entry get_pivot() {
        for (;;) {
            const Entry p = wc.get_pivot();
            if (p.idx != kNone || owed.empty()) return p;
            const uint32_t lo = front;
            front = owed_min > UINT32_MAX - grow ? UINT32_MAX : owed_min + grow;
            grow = grow > (UINT32_MAX >> 1) ? UINT32_MAX : 2 * grow;
            owed_min = UINT32_MAX;
            owed2.clear();
            for (const Entry& s : owed) push_window(s, lo, owed2);
            owed.swap(owed2);
        }
    }

    // Returns the pivot (idx kNone: the column cancelled out, an essential
    // class) and whether the emergent-pair shortcut paired it.
    std::pair<Entry, bool> reduce(const std::vector<Entry>& cols, uint64_t c, const PivotMap& pivots,
                                  const std::vector<uint64_t>& off, const std::vector<Entry>& red,
                                  const uint64_t* em_idx, const uint8_t* em_app) {
        const Entry col = cols[c];
        wc.reset(col.d, dmax);
        wr.clear();
        owed.clear();
        owed_min = UINT32_MAX;
        grow = std::max<uint32_t>(1, (top_bits > dbits(col.d) ? top_bits - dbits(col.d) : 0) >> TT_FRONT);
        // A graph complex pushes everything at once: a simplex has only its
        // common neighbours as cofacets, and a raise would repeat the row
        // walks that find them.
        front = hc.mat ? dbits(col.d) + grow : UINT32_MAX;
        if (em_idx) {
            // GPU-supplied first zero cofacet and its zero-apparent-facet flag
            if (em_idx[c] != kNone && !em_app[c] && pivots.find(em_idx[c]) == kNone)
                return {Entry{em_idx[c], col.d}, true};
            push_coboundary(col);
        } else {
            // the first cofacet with the column's diameter pairs it when no
            // earlier column owns it and it has no zero-apparent facet;
            // otherwise the whole coboundary goes into the queue
            uint32_t cv[34];
            cx.decode(col.idx, nv, vd);
            const uint64_t z = cx.zero_cofacet(vd, nv, col.d, cv);
            if (z != kNone && pivots.find(z) == kNone && cx.zero_apparent_facet(Entry{z, col.d}, nv + 1).idx == kNone)
                return {Entry{z, col.d}, true};
            push_coboundary(col);
        }
        Entry pivot = get_pivot();
        for (;;) {
            if (pivot.idx == kNone) return {pivot, false};
            const uint64_t j = pivots.find(pivot.idx);
            if (j != kNone) {
                wr.push_back(cols[j]);
                push_coboundary(cols[j]);
                for (uint64_t t = off[j]; t < off[j + 1]; ++t) {
                    wr.push_back(red[t]);
                    push_coboundary(red[t]);
                }
                pivot = get_pivot();
                continue;
            }
            // (a simplex with a zero-apparent facet is paired with that facet,
            // so it is never an owned pivot: the order of the two tests above
            // does not matter)
            const Entry fa = cx.zero_apparent_facet(pivot, nv + 1);
            if (fa.idx != kNone) {
                wr.push_back(fa);
                push_coboundary(fa);
                pivot = get_pivot();
                continue;
            }
            return {pivot, false};
        }
    }
};

// A column's reduction as one worker left it, waiting for its commit.
struct Pending {
    Entry pivot;
    bool emergent = false;
    std::vector<Entry> wr;
};

// Worker threads for the batch-parallel reduction: run(count, fn) calls
// fn(worker, i) for every i < count, spread over the workers and the caller.
struct Pool {
    std::vector<std::thread> th;
    std::mutex mu;
    std::condition_variable cv, done_cv;
    uint64_t gen = 0, count = 0;
    std::atomic<uint64_t> next{0};
    unsigned busy = 0;
    bool quit = false;
    std::function<void(unsigned, uint64_t)> fn;

    explicit Pool(unsigned workers) {
        for (unsigned w = 1; w <= workers; ++w)
            th.emplace_back([this, w] {
                uint64_t seen = 0;
                for (;;) {
                    {
                        std::unique_lock<std::mutex> l(mu);
                        cv.wait(l, [&] { return quit || gen != seen; });
                        if (quit) return;
                        seen = gen;
                    }
                    drain(w);
                    std::lock_guard<std::mutex> l(mu);
                    if (--busy == 0) done_cv.notify_one();
                }
            });
    }
    void drain(unsigned w) {
        for (uint64_t i; (i = next.fetch_add(1, std::memory_order_relaxed)) < count;) fn(w, i);
    }
    template <typename F>
    void run(uint64_t n, F&& f) {
        {
            std::lock_guard<std::mutex> l(mu);
            fn = std::forward<F>(f);
            count = n;
            next.store(0, std::memory_order_relaxed);
            busy = unsigned(th.size());
            ++gen;
        }
        cv.notify_all();
        drain(0);
        std::unique_lock<std::mutex> l(mu);
        done_cv.wait(l, [&] { return busy == 0; });
    }
    ~Pool() {
        {
            std::lock_guard<std::mutex> l(mu);
            quit = true;
        }
        cv.notify_all();
        for (auto& t : th) t.join();
    }
};

// compute_pairs' loop over the columns, with the same pivots, stored
// reductions and bars as the sequential algorithm.
//
// With several threads the columns go in batches. First every column of a
// batch is reduced in parallel against the pivots of the columns before the
// batch (read-only during the pass). Then the batch is committed in column
// order: a column whose result names a pivot that an earlier column of the
// same batch has just claimed (or whose emergent cofacet it claimed) is
// reduced again, now against every pivot before it. This gives the sequential
// result: until a reduction meets a simplex without an owner in the snapshot,
// every lookup it makes has the answer the sequential algorithm gets (a
// simplex has at most one owner, and one with a zero-apparent facet has
// none); an essential result or an unclaimed pivot is therefore final. The
// batch shrinks when such clashes are frequent and grows when they are rare.
template <class K>
Bars reduce_columns(const HostComplex& hc, const Binom& B, uint32_t dim, const std::vector<Entry>& cols,
                    const uint64_t* em_idx, const uint8_t* em_app, std::vector<uint64_t>& pivot_list,
                    ReduceStats& st, unsigned threads) {
    Bars bars;
    PivotMap pivots(cols.size() + 16);
    std::vector<uint64_t> off{0};
    std::vector<Entry> red;
    // the largest diameter an entry can have: the threshold, else the largest
    // distance of the complex
    float dmax = hc.thr;
    if (!(dmax < INFINITY)) {
        dmax = 0;
        const float* v = hc.mat ? hc.mat : hc.w;
        const uint64_t m = hc.mat ? uint64_t(hc.n) * hc.n : (hc.n ? hc.rp[hc.n] : 0);
        for (uint64_t i = 0; i < m; ++i)
            if (v[i] < INFINITY) dmax = std::max(dmax, v[i]);
    }
    auto commit = [&](uint64_t c, const Entry& pivot, bool emergent, std::vector<Entry>& wr) {
        const Entry col = cols[c];
        if (pivot.idx == kNone) {
            bars.birth.push_back(col.d);
            bars.death.push_back(INFINITY);
            bars.birth_idx.push_back(col.idx);
            bars.death_idx.push_back(kNone);
        } else if (emergent) {
            ++st.emergent;
            pivots.insert(pivot.idx, c);
        } else {
            if (pivot.d > col.d) {
                bars.birth.push_back(col.d);
                bars.death.push_back(pivot.d);
                bars.birth_idx.push_back(col.idx);
                bars.death_idx.push_back(pivot.idx);
            }
            pivots.insert(pivot.idx, c);
            std::sort(wr.begin(), wr.end(), precedes);
            for (size_t x = 0; x < wr.size();) {
                if (x + 1 < wr.size() && wr[x].idx == wr[x + 1].idx) x += 2;
                else red.push_back(wr[x++]);
            }
        }
        off.push_back(red.size());
    };
    std::vector<ColumnReducer<K>> workers;
    workers.reserve(std::max(1u, threads));
    workers.emplace_back(hc, B, dim, dmax);
    if (threads <= 1) {
        ColumnReducer<K>& w = workers[0];
        for (uint64_t c = 0; c < cols.size(); ++c) {
            const auto r = w.reduce(cols, c, pivots, off, red, em_idx, em_app);
            commit(c, r.first, r.second, w.wr);
        }
    } else {
        for (unsigned t = 1; t < threads; ++t) workers.emplace_back(hc, B, dim, dmax);
        Pool pool(threads - 1);
        std::vector<Pending> pend;
        uint64_t batch = 256;
        for (uint64_t c0 = 0; c0 < cols.size();) {
            const uint64_t nb = std::min<uint64_t>(batch, cols.size() - c0);
            if (pend.size() < nb) pend.resize(nb);
            pool.run(nb, [&](unsigned w, uint64_t i) {
                ColumnReducer<K>& r = workers[w];
                const auto res = r.reduce(cols, c0 + i, pivots, off, red, em_idx, em_app);
                pend[i].pivot = res.first;
                pend[i].emergent = res.second;
                pend[i].wr.swap(r.wr);
            });
            uint64_t clashes = 0;
            for (uint64_t i = 0; i < nb; ++i) {
                Pending& p = pend[i];
                if (p.pivot.idx != kNone && pivots.find(p.pivot.idx) != kNone) {
                    ++clashes;
                    const auto res = workers[0].reduce(cols, c0 + i, pivots, off, red, em_idx, em_app);
                    commit(c0 + i, res.first, res.second, workers[0].wr);
                } else {
                    commit(c0 + i, p.pivot, p.emergent, p.wr);
                }
            }
            c0 += nb;
            if (clashes * 16 > nb) batch = std::max<uint64_t>(32, batch / 2);
            else if (clashes * 64 < nb) batch = std::min<uint64_t>(1u << 16, batch * 2);
        }
    }
    st.columns = cols.size();
    pivot_list.clear();
    for (uint64_t s = 0; s < pivots.k.size(); ++s)
        if (pivots.k[s] != kNone) pivot_list.push_back(pivots.k[s]);
    std::sort(pivot_list.begin(), pivot_list.end());
    return bars;
}

}  // namespace

Bars compute_pairs(const HostComplex& hc, uint32_t dim, uint32_t maxdim, const std::vector<Entry>& cols,
                   const uint64_t* em_idx, const uint8_t* em_app, std::vector<uint64_t>& pivot_list,
                   ReduceStats& st, unsigned threads) {
    const Binom B(hc.n, maxdim + 2);
    // automatic: every hardware thread, for enough columns to pay for them
    if (threads == 0) threads = cols.size() < 4096 ? 1u : std::max(1u, std::thread::hardware_concurrency());
    // every cofacet index below 2^32: the packed queue keys
    if (B(hc.n, dim + 2) <= (uint64_t(1) << 32))
        return reduce_columns<PackedKey>(hc, B, dim, cols, em_idx, em_app, pivot_list, st, threads);
    return reduce_columns<WideKey>(hc, B, dim, cols, em_idx, em_app, pivot_list, st, threads);
}

std::vector<Entry> assemble(const HostComplex& hc, uint32_t dim, uint32_t maxdim,
                            const std::vector<Entry>& simplices, const std::vector<uint64_t>& pivots_sorted,
                            std::vector<Entry>* next, uint64_t* skipped, unsigned threads) {
    const Binom B(hc.n, maxdim + 2);
    const uint32_t nv = dim + 1;
    if (threads == 0) threads = std::max(1u, std::thread::hardware_concurrency());
    threads = unsigned(std::max<uint64_t>(1, std::min<uint64_t>(threads, simplices.size() / 256 + 1)));
    std::vector<std::vector<Entry>> cols(threads), nexts(threads);
    std::vector<uint64_t> skip(threads, 0);
    std::vector<std::string> errs(threads);
    auto work = [&](unsigned t) {
        try {
            const Cx cx{hc, B, {}, {}};
            uint32_t vd[34], cv[34];
            const uint64_t lo = simplices.size() * t / threads, hi = simplices.size() * (t + 1) / threads;
            for (uint64_t s = lo; s < hi; ++s) {
                cx.decode(simplices[s].idx, nv, vd);
                // the cofacets through a vertex above the simplex's largest
                // (t == 0): every simplex of the next dimension exactly once
                cx.cofacets(vd, nv, simplices[s].d, hc.thr, [&](const Entry& cf, uint32_t w, uint32_t tt) {
                    if (tt > 0) return false;
                    if (next) nexts[t].push_back(cf);
                    if (std::binary_search(pivots_sorted.begin(), pivots_sorted.end(), cf.idx)) return true;
                    cv[0] = w;
                    for (uint32_t i = 0; i < nv; ++i) cv[i + 1] = vd[i];
                    if (cx.in_zero_apparent_pair(cv, nv + 1, cf)) {
                        ++skip[t];
                        return true;
                    }
                    cols[t].push_back(cf);
                    return true;
                });
            }
        } catch (const std::exception& e) {
            errs[t] = e.what();
        }
    };
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < threads; ++t) pool.emplace_back(work, t);
    work(0);
    for (auto& th : pool) th.join();
    for (const auto& e : errs)
        if (!e.empty()) throw std::runtime_error(e);
    std::vector<Entry> out;
    uint64_t total = 0;
    for (const auto& v : cols) total += v.size();
    out.reserve(total);
    for (const auto& v : cols) out.insert(out.end(), v.begin(), v.end());
    std::sort(out.begin(), out.end(), [](const Entry& a, const Entry& b) { return precedes(b, a); });
    if (next) {
        next->clear();
        for (const auto& v : nexts) next->insert(next->end(), v.begin(), v.end());
    }
    if (skipped) {
        *skipped = 0;
        for (uint64_t x : skip) *skipped += x;
    }
    return out;
}

namespace {

inline uint64_t choose2(uint64_t v) { return v * (v - 1) / 2; }
inline uint64_t choose3(uint64_t v) { return uint64_t((unsigned __int128)v * (v - 1) * (v - 2) / 6); }

// Every triangle a > b > c of the graph complex: its edge (a, b) is the upper
// slot s of row a, (a, c) and (b, c) the slots pa of row a and pb of row b.
// fn(a, s, pa, pb, diameter). stop() is asked before each row: true ends the
// enumeration early.
template <typename F, typename S>
void for_each_triangle(const HostComplex& hc, F&& fn, S&& stop, uint32_t a0 = 0, uint32_t a1 = UINT32_MAX) {
    for (uint32_t a = a0; a < std::min(a1, hc.n) && !stop(); ++a)
        for (uint64_t s = hc.rp[a]; s < hc.rp[a + 1]; ++s) {
            const uint32_t b = hc.ci[s];
            if (b >= a) break;   // rows ascend: the upper slots come first
            if (!(hc.w[s] <= hc.thr)) continue;
            uint64_t pa = hc.rp[a], pb = hc.rp[b];
            const uint64_t ea = hc.rp[a + 1], eb = hc.rp[b + 1];
            while (pa < ea && pb < eb) {
                const uint32_t xa = hc.ci[pa], xb = hc.ci[pb];
                if (xa >= b || xb >= b) break;
                if (xa != xb) {
                    pa += xa < xb;
                    pb += xb < xa;
                    continue;
                }
                if (hc.w[pa] <= hc.thr && hc.w[pb] <= hc.thr)
                    fn(a, s, pa, pb, std::max(hc.w[s], std::max(hc.w[pa], hc.w[pb])));
                ++pa;
                ++pb;
            }
        }
}

}  // namespace

// f(t, i0, i1) on `threads` host threads over [0, n) in chunks of `chunk`
// handed out in order (each chunk to the next free thread).
template <typename F>
void parallel_chunks(unsigned threads, uint64_t n, uint64_t chunk, F&& f) {
    if (threads <= 1 || n <= chunk) {
        if (n) f(0u, uint64_t(0), n);
        return;
    }
    std::atomic<uint64_t> next{0};
    std::vector<std::thread> th;
    for (unsigned t = 0; t < threads; ++t)
        th.emplace_back([&, t] {
            for (uint64_t i; (i = next.fetch_add(chunk)) < n;) f(t, i, std::min(n, i + chunk));
        });
    for (auto& x : th) x.join();
}

// Sorts v by cmp on `threads` host threads: sorted runs, then rounds of
// pairwise merges (a total order: equal keys need no stability).
template <typename T, typename Cmp>
void parallel_sort(std::vector<T>& v, Cmp cmp, unsigned threads) {
    const size_t n = v.size();
    if (threads <= 1 || n < (size_t(1) << 16)) {
        std::sort(v.begin(), v.end(), cmp);
        return;
    }
    size_t parts = 1;
    while (parts < threads) parts <<= 1;
    std::vector<size_t> b(parts + 1);
    for (size_t i = 0; i <= parts; ++i) b[i] = n * i / parts;
    parallel_chunks(threads, parts, 1, [&](unsigned, uint64_t i0, uint64_t i1) {
        for (uint64_t i = i0; i < i1; ++i) std::sort(v.begin() + ptrdiff_t(b[i]), v.begin() + ptrdiff_t(b[i + 1]), cmp);
    });
    std::vector<T> tmp(n);
    for (size_t width = 1; width < parts; width <<= 1) {
        parallel_chunks(threads, parts / (2 * width), 1, [&](unsigned, uint64_t j0, uint64_t j1) {
            for (uint64_t j = j0; j < j1; ++j) {
                const size_t lo = b[2 * width * j], mid = b[2 * width * j + width], hi = b[2 * width * (j + 1)];
                std::merge(v.begin() + ptrdiff_t(lo), v.begin() + ptrdiff_t(mid), v.begin() + ptrdiff_t(mid),
                           v.begin() + ptrdiff_t(hi), tmp.begin() + ptrdiff_t(lo), cmp);
            }
        });
        v.swap(tmp);
    }
}

uint64_t graph_triangles(const HostComplex& hc, uint64_t limit) {
    uint64_t t = 0;
    for_each_triangle(hc, [&](uint32_t, uint64_t, uint64_t, uint64_t, float) { ++t; }, [&] { return t > limit; });
    return t;
}

// Boundary-matrix reduction of dimension 2 (the standard persistence
// algorithm: columns in filtration order, a column whose lowest entry, its
// latest edge, is owned by an earlier column adds that column). The
// filtration order is the reducer's (diameter ascending, larger index first
// among equal diameters), and the persistence pairing of one total order is
// unique, so an edge is paired with the same triangle as by compute_pairs.
// Edges that are never a lowest entry are essential; they cost nothing here,
// where the coboundary reducer cancels their whole coboundaries.
Bars graph_pairs_dim1(const HostComplex& hc, const std::vector<Entry>& cols, ReduceStats& st, bool* gave_up,
                      uint64_t max_store, uint64_t max_tris, unsigned threads) {
    if (gave_up) *gave_up = false;
    if (threads == 0) threads = std::max(1u, std::thread::hardware_concurrency());
    const uint32_t n = hc.n;
    const uint64_t nnz = n ? hc.rp[n] : 0;
    // kept edges by upper slot, ranked in filtration order (rows split over
    // the threads: per-row counts, offsets, then the edges in place)
    struct Edge {
        float d;
        uint64_t idx, slot;
    };
    std::vector<uint64_t> roff(uint64_t(n) + 1, 0);
    parallel_chunks(threads, n, 4096, [&](unsigned, uint64_t a0, uint64_t a1) {
        for (uint64_t a = a0; a < a1; ++a) {
            uint64_t c = 0;
            for (uint64_t s = hc.rp[a]; s < hc.rp[a + 1] && hc.ci[s] < a; ++s) c += hc.w[s] <= hc.thr;
            roff[a + 1] = c;
        }
    });
    for (uint32_t a = 0; a < n; ++a) roff[a + 1] += roff[a];
    std::vector<Edge> edges(roff[n]);
    parallel_chunks(threads, n, 4096, [&](unsigned, uint64_t a0, uint64_t a1) {
        for (uint64_t a = a0; a < a1; ++a) {
            uint64_t o = roff[a];
            for (uint64_t s = hc.rp[a]; s < hc.rp[a + 1] && hc.ci[s] < a; ++s)
                if (hc.w[s] <= hc.thr) edges[o++] = Edge{hc.w[s], choose2(a) + hc.ci[s], s};
        }
    });
    parallel_sort(edges, [](const Edge& x, const Edge& y) { return x.d < y.d || (x.d == y.d && x.idx > y.idx); },
                  threads);
    if (edges.size() >= UINT32_MAX) throw std::length_error("gb300: too many edges for the boundary reduction");
    std::vector<uint32_t> rank(nnz, UINT32_MAX);
    parallel_chunks(threads, edges.size(), 1 << 16, [&](unsigned, uint64_t r0, uint64_t r1) {
        for (uint64_t r = r0; r < r1; ++r) rank[edges[r].slot] = uint32_t(r);
    });
    // triangles in filtration order, each with its three edge ranks (rows
    // split over the threads; more than max_tris gives up)
    struct Tri {
        float d;
        uint64_t idx;
        uint32_t e[3];
    };
    std::vector<std::vector<Tri>> part(threads);
    std::atomic<uint64_t> total{0};
    std::atomic<bool> over{false};
    parallel_chunks(threads, n, 1024, [&](unsigned t, uint64_t a0, uint64_t a1) {
        if (over.load(std::memory_order_relaxed)) return;
        std::vector<Tri>& out = part[t];
        const size_t before = out.size();
        for_each_triangle(hc, [&](uint32_t a, uint64_t s, uint64_t pa, uint64_t pb, float d) {
            out.push_back(Tri{d, choose3(a) + choose2(hc.ci[s]) + hc.ci[pa], {rank[s], rank[pa], rank[pb]}});
        }, [] { return false; }, uint32_t(a0), uint32_t(a1));
        if (total.fetch_add(out.size() - before) + (out.size() - before) > max_tris) over.store(true);
    });
    if (over.load()) {
        if (!gave_up) throw std::length_error("gb300: too many triangles for the boundary reduction");
        *gave_up = true;
        return Bars{};
    }
    std::vector<Tri> tris;
    tris.reserve(total.load());
    for (auto& v : part) {
        tris.insert(tris.end(), v.begin(), v.end());
        std::vector<Tri>().swap(v);
    }
    parallel_sort(tris, [](const Tri& x, const Tri& y) { return x.d < y.d || (x.d == y.d && x.idx > y.idx); },
                  threads);
    if (tris.size() >= UINT32_MAX) throw std::length_error("gb300: too many triangles for the boundary reduction");
    // reduced columns (edge ranks, descending) stored back to back; with
    // gave_up, at most max_store entries (default 16 a triangle): past that
    // the fill-in of long reduction chains outgrows the coboundary
    // reducer's memory, and the caller reduces with compute_pairs instead
    if (gave_up && !max_store) max_store = 16 * uint64_t(tris.size()) + 4096;
    std::vector<uint32_t> owner(edges.size(), UINT32_MAX);   // edge rank -> triangle
    std::vector<uint64_t> off(tris.size() + 1, 0);
    std::vector<uint32_t> store;
    // Adds reduced columns to cur (descending edge ranks) while its lowest
    // entry has an owner.
    auto reduce = [&](std::vector<uint32_t>& cur, std::vector<uint32_t>& tmp) {
        while (!cur.empty() && owner[cur[0]] != UINT32_MAX) {
            const uint32_t o = owner[cur[0]];
            const uint32_t* q = store.data() + off[o];
            const uint32_t* qe = store.data() + off[o + 1];
            tmp.clear();
            size_t i = 0;
            while (i < cur.size() && q < qe) {
                if (cur[i] > *q) tmp.push_back(cur[i++]);
                else if (*q > cur[i]) tmp.push_back(*q++);
                else ++i, ++q;
            }
            tmp.insert(tmp.end(), cur.begin() + ptrdiff_t(i), cur.end());
            tmp.insert(tmp.end(), q, qe);
            cur.swap(tmp);
        }
    };
    std::vector<uint32_t> cur, tmp;
    for (uint32_t t = 0; t < tris.size(); ++t) {
        cur.assign(tris[t].e, tris[t].e + 3);
        std::sort(cur.begin(), cur.end(), std::greater<uint32_t>());
        reduce(cur, tmp);
        if (!cur.empty()) {
            owner[cur[0]] = t;
            store.insert(store.end(), cur.begin(), cur.end());
            if (gave_up && store.size() > max_store) {
                *gave_up = true;
                return Bars{};
            }
        }
        off[t + 1] = store.size();
    }
    // bars in column order, as compute_pairs emits them: each column's bar
    // found in parallel (0: none, 1: essential, 2: finite), then compacted
    std::vector<uint8_t> kind(cols.size(), 0);
    std::vector<uint32_t> dtri(cols.size(), UINT32_MAX);
    std::atomic<int> bad{0};
    parallel_chunks(threads, cols.size(), 4096, [&](unsigned, uint64_t c0, uint64_t c1) {
        for (uint64_t ci = c0; ci < c1; ++ci) {
            const Entry& c = cols[ci];
            uint32_t u = uint32_t((1.0 + std::sqrt(1.0 + 8.0 * double(c.idx))) / 2.0);
            while (choose2(u) > c.idx) --u;
            while (choose2(u + 1) <= c.idx) ++u;
            const uint32_t v = uint32_t(c.idx - choose2(u));
            const uint32_t* b = hc.ci + hc.rp[u];
            const uint32_t* e = hc.ci + hc.rp[u + 1];
            const uint32_t* it = std::lower_bound(b, e, v);
            if (it == e || *it != v) {
                bad.store(1);
                continue;
            }
            const uint32_t r = rank[uint64_t(it - hc.ci)];
            if (r == UINT32_MAX) {
                bad.store(2);
                continue;
            }
            const uint32_t t = owner[r];
            if (t == UINT32_MAX) kind[ci] = 1;
            else if (tris[t].d > c.d) kind[ci] = 2, dtri[ci] = t;
        }
    });
    if (bad.load() == 1) throw std::logic_error("gb300: a column's edge is not in the graph");
    if (bad.load() == 2) throw std::logic_error("gb300: a column's edge is above the threshold");
    Bars bars;
    for (size_t ci = 0; ci < cols.size(); ++ci) {
        if (!kind[ci]) continue;
        const Entry& c = cols[ci];
        bars.birth.push_back(c.d);
        bars.birth_idx.push_back(c.idx);
        if (kind[ci] == 1) {
            bars.death.push_back(INFINITY);
            bars.death_idx.push_back(kNone);
        } else {
            bars.death.push_back(tris[dtri[ci]].d);
            bars.death_idx.push_back(tris[dtri[ci]].idx);
        }
    }
    st.columns = cols.size();
    st.emergent = 0;
    return bars;
}

}  // namespace host
}  // namespace tt
