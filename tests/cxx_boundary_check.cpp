// cxx_boundary_check.cpp — the C++ boundary, compiled for real: this
// translation unit includes the UNMODIFIED reference headers and
// include/turbotops_gb300.hpp, links libturbotops_gb300.so, and compares the
// GB300 glue with the reference's own functions on the same inputs:
//
//   tops::gb300::persistence(points, ...)  vs tops::persistence(points, ...)
//   tops::gb300::persistence(CsrGraph, ...) vs tops::persistence(CsrGraph, ...)
//   tops::gb300::knn_graph_exact            vs knn_graph(c, knn_lists_exact(c, k))
//   tops::gb300::mst_h0                     vs mst::h0
//
// and the exception class and message of invalid inputs. Bars are compared
// per dimension in canonical (birth, death) order, bit for bit, as the
// reference CLI writes them. Prints "ok <checks>" and exits 0, or the first
// difference and exits 1. Built and run by tests/test_gpu_cxx_boundary.py.
#include "turbotops_gb300.hpp"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <functional>
#include <random>
#include <vector>

using namespace tops;

namespace {

int checks = 0;

[[noreturn]] void fail(const std::string& what) {
    std::printf("FAIL %s\n", what.c_str());
    std::exit(1);
}

std::vector<f32> cloud(u32 n, u32 dim, u32 seed, bool lattice = false) {
    std::mt19937 rng(seed);
    std::normal_distribution<f32> N(0.0f, 1.0f);
    std::uniform_int_distribution<int> U(0, 5);
    std::vector<f32> x(u64(n) * dim);
    for (auto& v : x) v = lattice ? f32(U(rng)) : N(rng);
    return x;
}

std::vector<std::pair<u32, u32>> canon(const rips::Barcode& b, u32 d) {
    std::vector<std::pair<u32, u32>> v;
    if (d >= b.ndims()) return v;
    for (u64 i = 0; i < b.birth[d].size(); ++i) {
        u32 x, y;
        std::memcpy(&x, &b.birth[d][i], 4);
        std::memcpy(&y, &b.death[d][i], 4);
        v.emplace_back(x, y);
    }
    std::sort(v.begin(), v.end(), [](auto a, auto b) {
        f32 ab, ad, bb, bd;
        std::memcpy(&ab, &a.first, 4), std::memcpy(&ad, &a.second, 4);
        std::memcpy(&bb, &b.first, 4), std::memcpy(&bd, &b.second, 4);
        return ab != bb ? ab < bb : (ad != bd ? ad < bd : a < b);
    });
    return v;
}

void same_bars(const rips::Barcode& ref, const rips::Barcode& got, u32 maxdim, const std::string& tag) {
    for (u32 d = 0; d <= maxdim; ++d) {
        if (canon(ref, d) != canon(got, d))
            fail(tag + ": H" + std::to_string(d) + " differs (" + std::to_string(canon(ref, d).size()) + " vs " +
                 std::to_string(canon(got, d).size()) + " bars)");
        ++checks;
    }
}

void same_result(const Result& ref, const Result& got, u32 maxdim, const std::string& tag) {
    same_bars(ref.barcode, got.barcode, maxdim, tag);
    if (std::memcmp(&ref.stats.threshold, &got.stats.threshold, 4) != 0)
        fail(tag + ": threshold " + std::to_string(ref.stats.threshold) + " vs " + std::to_string(got.stats.threshold));
    ++checks;
    // the same engine as the reference's mode auto; where that is RedZeD, the
    // reference's own engine ran on the GPU's edge list, so even the
    // discovery order of the bars and the edge count agree
    if (ref.stats.engine != got.stats.engine)
        fail(tag + ": engine " + ref.stats.engine + " vs " + got.stats.engine);
    ++checks;
    if (ref.stats.engine == "boundary") {
        for (u32 d = 0; d <= maxdim; ++d)
            if (ref.barcode.birth[d] != got.barcode.birth[d] || ref.barcode.death[d] != got.barcode.death[d])
                fail(tag + ": RedZeD bar order differs in H" + std::to_string(d));
        if (ref.stats.edges != got.stats.edges) fail(tag + ": edge count differs");
        ++checks;
    }
}

template <typename E>
void same_throw(const std::function<void()>& ref, const std::function<void()>& got, const std::string& tag) {
    std::string a = "<none>", b = "<none>";
    try { ref(); } catch (const E& e) { a = e.what(); } catch (...) { a = "<other type>"; }
    try { got(); } catch (const E& e) { b = e.what(); } catch (...) { b = "<other type>"; }
    if (a == "<none>" || a != b) fail(tag + ": reference '" + a + "' vs gb300 '" + b + "'");
    ++checks;
}

}  // namespace

int main() {
    // dense full Rips, maxdim 2 and 1, every metric
    for (const char* metric : {"l2", "l1", "linf", "lp:1.5"}) {
        const auto x = cloud(180, 3, 7);
        Options o;
        o.maxdim = 2;
        o.metric = metric;
        same_result(persistence(x.data(), 180, 3, o), gb300::persistence(x.data(), 180, 3, o), 2,
                    std::string("dense maxdim 2 ") + metric);
    }
    {
        const auto x = cloud(300, 4, 8, true);   // lattice: ties
        Options o;
        o.maxdim = 1;
        o.metric = "linf";
        same_result(persistence(x.data(), 300, 4, o), gb300::persistence(x.data(), 300, 4, o), 1, "dense ties");
    }
    // dense full Rips maxdim 1: mode auto's RedZeD, fed with the GPU's matrix and edges
    for (const char* metric : {"l2", "l1", "lp:1.5"}) {
        const auto x = cloud(700, 3, 12);
        Options o;
        o.metric = metric;
        same_result(persistence(x.data(), 700, 3, o), gb300::persistence(x.data(), 700, 3, o), 1,
                    std::string("dense redzed ") + metric);
    }
    // the device's leftover-coface predicate bits against their definition
    for (const char* metric : {"l2", "linf"}) {
        const auto x = cloud(333, 3, 14, std::string(metric) == "linf");
        const Metric mt = Metric::parse(metric);
        const u32 n = 333, words = (n + 63) / 64;
        std::vector<f32> mat(u64(n) * n), diam(u64(n) * n);
        std::vector<int32_t> verts(2 * u64(n) * n);
        std::vector<uint64_t> bits(u64(n) * words);
        f32 thr = INFINITY;
        u64 count = 0;
        gb300::check(tt_dense_redzed_pred_h(gb300::ctx(), x.data(), n, 3, int(mt.kind), mt.p, &thr, mat.data(),
                                            diam.data(), verts.data(), diam.size(), &count, bits.data()),
                     gb300::ctx());
        u64 set = 0;
        for (u32 u = 0; u < n; ++u)
            for (u32 v = u + 1; v < n; ++v) {
                const f32 d = mat[u64(u) * n + v];
                bool want = false;
                if (d <= thr)
                    for (u32 w = 0; w < n && !want; ++w) {
                        if (w == u || w == v) continue;
                        const f32 du = mat[u64(u) * n + w], dv = mat[u64(v) * n + w];
                        want = du <= d && dv <= d && (w < u || (w < v ? dv < d : (du < d && dv < d)));
                    }
                const bool got = (bits[u64(u) * words + (v >> 6)] >> (v & 63)) & 1u;
                if (got != want) fail(std::string("leftover predicate bit differs (") + metric + ")");
                set += got;
            }
        if (!set) fail("leftover predicate: no bit set");
        ++checks;
    }
    // a kNN graph of mean degree >= 16: RedZeD on the graph
    {
        const auto x = cloud(3000, 8, 13);
        Options o;
        o.graph = Options::Graph::Knn;
        o.k = 14;
        same_result(persistence(x.data(), 3000, 8, o), gb300::persistence(x.data(), 3000, 8, o), 1, "knn redzed");
    }
    // more than 131072 vertices: edge indices beyond the packed keys' 33 bits
    // (wide edge keys on the device), RedZeD's graph engine (k = 15) and the
    // library's own reduction (k = 6)
    {
        const u32 n = 140000;
        const auto x = cloud(n, 3, 15);
        for (const u32 k : {15u, 6u}) {
            Options o;
            o.graph = Options::Graph::Knn;
            o.k = k;
            same_result(persistence(x.data(), n, 3, o), gb300::persistence(x.data(), n, 3, o), 1,
                        "knn n = 140000, k = " + std::to_string(k));
        }
    }
    // kNN flag complex (L2 in R^32: the tensor-core filter path; lp:1.5), radius graph, MST
    {
        const auto x = cloud(2000, 32, 9);
        Options o;
        o.graph = Options::Graph::Knn;
        o.k = 12;
        same_result(persistence(x.data(), 2000, 32, o), gb300::persistence(x.data(), 2000, 32, o), 1, "knn l2");
        o.metric = "lp:1.5";
        same_result(persistence(x.data(), 2000, 32, o), gb300::persistence(x.data(), 2000, 32, o), 1, "knn lp");
        const PointCloud pc{x.data(), 2000, 32, Metric::parse("l2")};
        const CsrGraph a = knn_graph(pc, knn_lists_exact(pc, 12));
        const CsrGraph b = gb300::knn_graph_exact(pc, 12);
        if (a.row_ptr != b.row_ptr || a.col_idx != b.col_idx || a.m != b.m ||
            std::memcmp(a.weights.data(), b.weights.data(), 4 * a.weights.size()) != 0)
            fail("knn_graph_exact differs");
        ++checks;
        same_result(persistence(a, 1), gb300::persistence(a, 1), 1, "CsrGraph");
        same_result(persistence(a, 1, 4.0f), gb300::persistence(a, 1, 4.0f), 1, "CsrGraph threshold");
        same_bars(mst::h0(pc), gb300::mst_h0(pc), 0, "mst");
        same_bars(mst::h0(pc, 3.5f), gb300::mst_h0(pc, 3.5f), 0, "mst threshold");
    }
    {
        const auto x = cloud(600, 3, 10);
        Options o;
        o.threshold = 0.6f;
        same_result(persistence(x.data(), 600, 3, o), gb300::persistence(x.data(), 600, 3, o), 1, "radius");
        o.threshold = INFINITY;
        o.maxdim = 0;
        same_result(persistence(x.data(), 600, 3, o), gb300::persistence(x.data(), 600, 3, o), 0, "maxdim 0");
    }
    // invalid inputs: same exception class, same message
    {
        auto x = cloud(50, 3, 11);
        Options bad_metric;
        bad_metric.metric = "cosine";
        same_throw<std::invalid_argument>([&] { persistence(x.data(), 50, 3, bad_metric); },
                                          [&] { gb300::persistence(x.data(), 50, 3, bad_metric); }, "metric");
        Options bad_p;
        bad_p.metric = "lp:0.5";
        same_throw<std::invalid_argument>([&] { persistence(x.data(), 50, 3, bad_p); },
                                          [&] { gb300::persistence(x.data(), 50, 3, bad_p); }, "p < 1");
        Options bad_t;
        bad_t.threshold = -1.0f;
        same_throw<std::invalid_argument>([&] { persistence(x.data(), 50, 3, bad_t); },
                                          [&] { gb300::persistence(x.data(), 50, 3, bad_t); }, "threshold");
        Options bad_k;
        bad_k.graph = Options::Graph::Knn;
        bad_k.k = 0;
        same_throw<std::invalid_argument>([&] { persistence(x.data(), 50, 3, bad_k); },
                                          [&] { gb300::persistence(x.data(), 50, 3, bad_k); }, "k");
        // make_dense's memory budget: 50 points need 4900 bytes of lower triangle
        for (const Mode mode : {Mode::Auto, Mode::Coboundary}) {
            Options small;
            small.memory_budget = 4899;
            small.mode = mode;
            same_throw<std::length_error>([&] { persistence(x.data(), 50, 3, small); },
                                          [&] { gb300::persistence(x.data(), 50, 3, small); }, "memory budget");
            small.memory_budget = 4900;
            same_result(persistence(x.data(), 50, 3, small), gb300::persistence(x.data(), 50, 3, small), 1,
                        "budget just enough");
        }
        {
            Options small;
            small.memory_budget = 4899;
            const std::vector<const f32*> clouds{x.data()};
            const std::vector<u32> sizes{50};
            same_throw<std::length_error>([&] { persistence(x.data(), 50, 3, small); },
                                          [&] { gb300::persistence_batch(clouds, sizes, 3, small); },
                                          "memory budget, batch");
        }
        x[17] = NAN;
        Options o;
        same_throw<std::invalid_argument>([&] { persistence(x.data(), 50, 3, o); },
                                          [&] { gb300::persistence(x.data(), 50, 3, o); }, "non-finite");
        CsrGraph g;
        g.n = 3;
        g.m = 1;
        g.row_ptr = {0, 1, 1, 2};
        g.col_idx = {1, 0};          // (0, 1) and (2, 0): not symmetric
        g.weights = {1.0f, 1.0f};
        same_throw<std::invalid_argument>([&] { persistence(g, 1); }, [&] { gb300::persistence(g, 1); }, "graph");
    }
    std::printf("ok %d\n", checks);
    return 0;
}
