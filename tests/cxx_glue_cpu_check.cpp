// cxx_glue_cpu_check.cpp — the mechanism include/turbotops_gb300.hpp uses to
// feed the reference's RedZeD engine with edge lists built elsewhere, checked
// on the CPU: the engine (redzed::detail::run, unmodified) must call the
// glue's build_edges overload for the GpuEdges* geometries, and a prebuilt
// list equal to the reference's own gives the reference's diagram, bar for
// bar and in the same order. Here the prebuilt lists come from the
// reference's own build_edges, so no GPU is involved; the GPU test
// (cxx_boundary_check.cpp) feeds lists the device built.
#include <cstdio>
#include <cstring>
#include <random>

#include "turbotops_gb300.hpp"

using namespace tops;

namespace {
int overload_calls = 0;
}

// counts the handovers (the glue's overloads are found by argument-dependent
// lookup; a wrapper type here proves the engine takes that route)
namespace tops::gb300 {
struct CountingDense : GpuEdgesDense {
    using GpuEdgesDense::GpuEdgesDense;
};
inline void build_edges(const CountingDense& geo, redzed::detail::value_t t, const redzed::detail::BinomialTable& b,
                        redzed::detail::EdgeList& out) {
    ++overload_calls;
    build_edges(static_cast<const GpuEdgesDense&>(geo), t, b, out);
}
}  // namespace tops::gb300

// RedZeD's leftover-coface predicate per edge, from its definition (the
// device computes the same bits): some w != u, v within d(u, v) of both, with
// w < u, or u < w < v and d(w, v) < d, or w > v and both strictly shorter.
static std::vector<uint64_t> leftover_bits(const rips::DenseComplex& cx) {
    const u32 n = cx.n, words = (n + 63) / 64;
    std::vector<uint64_t> bits(size_t(n) * words, 0);
    for (u32 u = 0; u < n; ++u)
        for (u32 v = u + 1; v < n; ++v) {
            const f32 d = cx.dist(u, v);
            if (!(d <= cx.threshold)) continue;
            for (u32 w = 0; w < n; ++w) {
                if (w == u || w == v) continue;
                const f32 du = cx.dist(u, w), dv = cx.dist(v, w);
                if (!(du <= d && dv <= d)) continue;
                if (w < u || (w < v ? dv < d : (du < d && dv < d))) {
                    bits[size_t(u) * words + (v >> 6)] |= uint64_t(1) << (v & 63);
                    break;
                }
            }
        }
    return bits;
}

// The glue geometry with every predicate answer it gives from the bits
// checked against the reference's own scan.
namespace tops::gb300 {
struct CheckedDense : GpuEdgesDense {
    using GpuEdgesDense::GpuEdgesDense;
    mutable long answered = 0, wrong = 0;
    template <class Ready>
    bool any_common_radius_neighbor(const int32_t* xv, int m, size_t r, const std::vector<uint64_t>& sb,
                                    const std::vector<char>& seen, Ready&& ready) const {
        const bool mine = GpuEdgesDense::any_common_radius_neighbor(xv, m, r, sb, seen, ready);
        bool none = true;
        for (uint64_t w : sb) none = none && w == 0;
        if (m == 2 && none && leftover) {
            ++answered;
            wrong += mine != redzed::detail::DenseGeom::any_common_radius_neighbor(xv, m, r, sb, seen, ready);
        }
        return mine;
    }
};
inline void build_edges(const CheckedDense& geo, redzed::detail::value_t t, const redzed::detail::BinomialTable& b,
                        redzed::detail::EdgeList& out) {
    build_edges(static_cast<const GpuEdgesDense&>(geo), t, b, out);
}
}  // namespace tops::gb300

static bool same(const rips::Barcode& a, const rips::Barcode& b) {
    if (a.ndims() != b.ndims()) return false;
    for (u32 d = 0; d < a.ndims(); ++d) {
        if (a.birth[d].size() != b.birth[d].size()) return false;
        if (std::memcmp(a.birth[d].data(), b.birth[d].data(), 4 * a.birth[d].size()) ||
            std::memcmp(a.death[d].data(), b.death[d].data(), 4 * a.death[d].size()))
            return false;
    }
    return true;
}

int main() {
    int checks = 0;
    for (u32 seed = 1; seed <= 4; ++seed) {
        std::mt19937 rng(seed);
        std::normal_distribution<f32> N(0.0f, 1.0f);
        const u32 n = 150 + 40 * seed, dim = seed == 4 ? 4 : 3;
        std::vector<f32> x(u64(n) * dim);
        for (auto& v : x) v = seed == 4 ? f32(int(4 * N(rng))) : N(rng);   // seed 4: integer ties
        const PointCloud pc{x.data(), n, dim, Metric::parse(seed == 3 ? "l1" : "l2")};
        rips::DenseComplex cx = rips::make_dense(n, pc);
        cx.threshold = cx.enclosing_radius();
        const rips::Barcode ref = redzed::compute(cx, 1);
        redzed::detail::DenseGeom plain(cx);
        redzed::detail::BinomialTable bt(int(n) + 1, 3);
        redzed::detail::EdgeList el;
        redzed::detail::build_edges(plain, cx.threshold, bt, el);
        const int before = overload_calls;
        gb300::CountingDense geo(cx, &el);
        const rips::Barcode got = redzed::detail::run(geo, 1, cx.threshold);
        if (overload_calls != before + 1) { std::printf("FAIL overload not taken (seed %u)\n", seed); return 1; }
        if (!same(ref, got)) { std::printf("FAIL dense diagram differs (seed %u)\n", seed); return 1; }
        ++checks;
        // the leftover-coface predicate answered from precomputed bits
        {
            const std::vector<uint64_t> bits = leftover_bits(cx);
            redzed::detail::EdgeList el2;
            redzed::detail::build_edges(plain, cx.threshold, bt, el2);
            gb300::CheckedDense cgeo(cx, &el2, &bits);
            const rips::Barcode got2 = redzed::detail::run(cgeo, 1, cx.threshold);
            if (cgeo.answered == 0 || cgeo.wrong != 0) {
                std::printf("FAIL predicate answered %ld, wrong %ld (seed %u)\n", cgeo.answered, cgeo.wrong, seed);
                return 1;
            }
            if (!same(ref, got2)) { std::printf("FAIL diagram with the predicate differs (seed %u)\n", seed); return 1; }
            ++checks;
        }
        // sparse: a kNN graph
        const CsrGraph g = knn_graph(pc, knn_lists_exact(pc, 10));
        const rips::Barcode sref = redzed::compute_graph(g, 1);
        redzed::detail::SparseGeom<uint32_t> sp(g);
        redzed::detail::EdgeList sel;
        redzed::detail::build_edges(sp, INFINITY, bt, sel);
        gb300::GpuEdgesSparse<uint32_t> sgeo(g, &sel);
        if (!same(sref, redzed::detail::run(sgeo, 1, INFINITY))) {
            std::printf("FAIL sparse diagram differs (seed %u)\n", seed);
            return 1;
        }
        ++checks;
    }
    std::printf("ok %d\n", checks);
    return 0;
}
