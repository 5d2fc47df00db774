// turbotops_gb300.hpp — C++ glue that puts the GB300 front end behind the
// reference's own C++ types (dnbaker/turbotops v0.1.0, include/turbotops).
//
// Include it after (or instead of) "turbotops/turbotops.hpp" and link
// libturbotops_gb300.so (turbotops_gb300/_lib, built by
// `python -m turbotops_gb300.build`). Every function here has the signature of
// the reference function it stands in for, takes and returns the reference's
// types (PointCloud, Options, CsrGraph, Result, rips::Barcode) and throws the
// reference's exception types with the reference's messages: the C-ABI's
// statuses map back as TT_ERR_INVALID -> std::invalid_argument,
// TT_ERR_OVERFLOW -> std::overflow_error, TT_ERR_LENGTH -> std::length_error,
// anything else -> std::runtime_error.
//
//   tops::gb300::persistence(points, n, dim, Options)   turbotops.hpp:211-303
//   tops::gb300::persistence(CsrGraph, maxdim, ...)     turbotops.hpp:179-207
//   tops::gb300::knn_graph_exact(PointCloud, k)         graph.hpp:211-225 + :286-304
//   tops::gb300::mst_h0(PointCloud, threshold)          mst.hpp:25-99
//   tops::gb300::redzed_dense / redzed_graph            redzed.hpp:1433-1460
//   tops::gb300::persistence_batch(clouds, sizes, ...)  persistence() once per cloud
//
// Engines, as the reference's mode auto picks them (turbotops.hpp:121-162):
// H1 of dense full Rips and of graphs of mean degree >= 16 goes to the
// reference's own RedZeD engine (redzed::detail::run) on the host, fed with
// what the GPU built — the distance matrix and the sorted edge list
// (tt_dense_redzed_h / tt_graph_redzed_h) replace make_dense and
// build_edges, through the build_edges overloads below that the engine finds
// by argument-dependent lookup; everything else runs the library's own
// pipeline (GPU front end, host cohomology reduction, tt_persistence_h).
//
// One library context per calling thread (device 0, the legacy default
// stream), created on first use and destroyed at thread exit. The results
// are the reference's bit for bit (bars, thresholds, edge counts); the bar
// order within a dimension is this implementation's discovery order (the
// reference's depends on the engine its mode picks; its CLI and tests compare
// canonical order), and Stats' column/apparent/emergent counts describe this
// implementation's reduction.
#ifndef TURBOTOPS_GB300_HPP
#define TURBOTOPS_GB300_HPP

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <limits>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "turbotops/turbotops.hpp"
#include "turbotops_gb300.h"

namespace tops::gb300 {

inline tt_ctx* ctx() {
    thread_local struct Holder {
        tt_ctx* c = nullptr;
        Holder() {
            if (tt_ctx_create(0, nullptr, &c) != TT_OK) throw std::runtime_error(tt_last_error(nullptr));
        }
        ~Holder() { tt_ctx_destroy(c); }
    } h;
    return h.c;
}

// Status -> the reference's exception class, with the library's message.
inline void check(int st, const tt_ctx* c) {
    if (st == TT_OK) return;
    const std::string m = tt_last_error(c);
    if (st == TT_ERR_INVALID) throw std::invalid_argument(m);
    if (st == TT_ERR_OVERFLOW) throw std::overflow_error(m);
    if (st == TT_ERR_LENGTH) throw std::length_error(m);
    throw std::runtime_error(m);
}

// tt_barcode (library-owned) -> Result; frees the tt_barcode.
inline Result to_result(tt_barcode* b, u32 maxdim) {
    struct Free {
        tt_barcode* b;
        ~Free() { tt_barcode_free(b); }
    } guard{b};
    Result r;
    u64 o = 0;
    for (u32 d = 0; d < b->ndims; ++d) {
        r.barcode.ensure(d);
        for (u64 i = 0; i < b->count[d]; ++i) r.barcode.add(d, b->birth[o + i], b->death[o + i]);
        o += b->count[d];
    }
    r.barcode.ensure(maxdim);
    r.stats.method = b->method;
    r.stats.engine = r.stats.method == "mst" ? "mst" : "coboundary";
    r.stats.mode_reason = "gb300: GPU front end, host cohomology reduction";
    r.stats.threshold = b->threshold;
    r.stats.edges = b->edges;
    for (u32 d = 1; d < b->ndims && d < 32; ++d) {
        r.stats.columns.push_back(b->columns[d - 1]);
        r.stats.apparent.push_back(b->apparent[d - 1]);
        r.stats.emergent.push_back(b->emergent[d - 1]);
    }
    return r;
}

inline CsrGraph knn_graph_exact(const PointCloud& pc, u32 k);
inline CsrGraph radius_graph(const PointCloud& pc, f32 tau);

// ---- RedZeD on the host, fed by the GPU -------------------------------------
// The reference's geometry policies with the edge list already built on the
// GPU: Engine::run calls build_edges(geo, ...) unqualified, and for these
// types the overloads below (found by argument-dependent lookup, preferred as
// non-templates) hand over the prebuilt list instead of running the host pass.
struct GpuEdgesDense : redzed::detail::DenseGeom {
    redzed::detail::EdgeList* prebuilt;
    // RedZeD's static leftover-coface predicate per kept edge, from the GPU
    // (tt_dense_redzed_pred_h): n x ceil(n / 64) words, or null
    const std::vector<uint64_t>* leftover = nullptr;
    GpuEdgesDense(const rips::DenseComplex& cx, redzed::detail::EdgeList* e,
                  const std::vector<uint64_t>* left = nullptr)
        : DenseGeom(cx), prebuilt(e), leftover(left) {}
    // has_leftover_coface's scan (redzed.hpp:728-765): for an edge with no
    // vertex excluded (no seen bit), the GPU's answer; otherwise the
    // reference's own scan. The engine asks only about cycle-closing edges at
    // maxdim 1 with the radius graph grown to the edge's length, which is the
    // predicate's definition.
    template <class Ready>
    bool any_common_radius_neighbor(const int32_t* xv, int m, size_t r, const std::vector<uint64_t>& seenbits,
                                    const std::vector<char>& seen, Ready&& ready) const {
        if (leftover && m == 2) {
            bool none = true;
            for (size_t w = 0; w < seenbits.size() && none; ++w) none = seenbits[w] == 0;
            if (none) {
                const size_t words = size_t(words_of(n));
                return ((*leftover)[size_t(xv[0]) * words + size_t(xv[1] >> 6)] >> (xv[1] & 63)) & 1u;
            }
        }
        return DenseGeom::any_common_radius_neighbor(xv, m, r, seenbits, seen, std::forward<Ready>(ready));
    }
    static int words_of(int n) { return (n + 63) / 64; }
};
template <typename Rank>
struct GpuEdgesSparse : redzed::detail::SparseGeom<Rank> {
    redzed::detail::EdgeList* prebuilt;
    GpuEdgesSparse(const CsrGraph& g, redzed::detail::EdgeList* e) : redzed::detail::SparseGeom<Rank>(g), prebuilt(e) {}
};
inline void build_edges(const GpuEdgesDense& geo, redzed::detail::value_t, const redzed::detail::BinomialTable&,
                        redzed::detail::EdgeList& out) {
    out = std::move(*geo.prebuilt);
}
template <typename Rank>
inline void build_edges(const GpuEdgesSparse<Rank>& geo, redzed::detail::value_t,
                        const redzed::detail::BinomialTable&, redzed::detail::EdgeList& out) {
    out = std::move(*geo.prebuilt);
}

// redzed::compute over make_dense(points) cut at the threshold (+inf: the
// enclosing radius), the matrix and the edge list from the GPU, and at
// maxdim 1 the leftover-coface predicate too (unless device_predicate is off).
inline rips::Barcode redzed_dense(const f32* points, u32 n, u32 dim, const Metric& m, u32 maxdim, f32 threshold,
                                  u64* edges = nullptr, f32* thr_out = nullptr, bool device_predicate = true) {
    tt_ctx* c = ctx();
    rips::DenseComplex cx;
    cx.n = n;
    cx.full = true;
    cx.mat.resize(u64(n) * n);
    redzed::detail::EdgeList el;
    const u64 cap = n > 1 ? u64(n) * (n - 1) / 2 : 0;
    el.diam.resize(cap);
    el.verts.resize(2 * cap);
    f32 thr = threshold;
    u64 count = 0;
    const bool pred = device_predicate && maxdim == 1;
    std::vector<uint64_t> left(pred ? size_t(n) * size_t((n + 63) / 64) : 0);
    check(tt_dense_redzed_pred_h(c, points, n, dim, int(m.kind), m.p, &thr, cx.mat.data(), el.diam.data(),
                                 el.verts.data(), cap, &count, pred ? left.data() : nullptr),
          c);
    el.count = count;
    el.diam.resize(count);
    el.verts.resize(2 * count);
    cx.threshold = thr;
    if (thr_out) *thr_out = thr;
    GpuEdgesDense geo(cx, &el, pred ? &left : nullptr);
    return redzed::detail::run(geo, maxdim, cx.threshold, edges);
}

// redzed::compute_graph (redzed.hpp:1450-1460), the edge list from the GPU.
inline rips::Barcode redzed_graph(const CsrGraph& g, u32 maxdim, f32 threshold = INFINITY, u64* edges = nullptr) {
    tt_ctx* c = ctx();
    redzed::detail::EdgeList el;
    el.diam.resize(g.m);
    el.verts.resize(2 * g.m);
    u64 count = 0;
    check(tt_graph_redzed_h(c, g.row_ptr.data(), g.col_idx.data(), g.weights.data(), g.n, threshold, el.diam.data(),
                            el.verts.data(), g.m, &count),
          c);
    el.count = count;
    el.diam.resize(count);
    el.verts.resize(2 * count);
    if (g.m < u64(std::numeric_limits<uint32_t>::max())) {
        GpuEdgesSparse<uint32_t> geo(g, &el);
        return redzed::detail::run(geo, maxdim, threshold, edges);
    }
    GpuEdgesSparse<uint64_t> geo(g, &el);
    return redzed::detail::run(geo, maxdim, threshold, edges);
}

inline Result redzed_result(rips::Barcode&& b, u32 maxdim, const char* method, const std::string& why, f32 thr,
                            u64 edges) {
    Result r;
    r.barcode = std::move(b);
    r.barcode.ensure(maxdim);
    r.stats.method = method;
    r.stats.engine = "boundary";
    r.stats.mode_reason = why;
    r.stats.threshold = thr;
    r.stats.edges = edges;
    return r;
}

// tops::persistence(points, n, dim, Options) (turbotops.hpp:211-303).
inline Result persistence(const f32* points, u32 n, u32 dim, const Options& o) {
    const auto t0 = std::chrono::steady_clock::now();
    if (o.approximate)
        throw std::invalid_argument("persistence: approximate kNN (HNSW) is not offered by the GB300 front end");
    tt_ctx* c = ctx();
    check(tt_ctx_set_memory_budget(c, o.memory_budget), c);   // make_dense's budget (rips.hpp:383-416)
    int kind = 0;
    float p = 2.0f;
    check(tt_metric_parse(o.metric.c_str(), &kind, &p), nullptr);
    detail::validate_options(o.threshold, o.graph == Options::Graph::Knn ? o.k : 1);
    const bool dense = o.graph == Options::Graph::Full && std::isinf(o.threshold) && o.maxdim > 0;
    if (o.graph == Options::Graph::Full && !std::isinf(o.threshold) && o.maxdim > 0) {
        // radius graph: the reference builds it, then picks the engine by mean degree
        const auto tg = std::chrono::steady_clock::now();
        const CsrGraph g = gb300::radius_graph(PointCloud{points, n, dim, Metric::minkowski(p)}, o.threshold);
        const double sg = std::chrono::duration<double>(std::chrono::steady_clock::now() - tg).count();
        std::string why;
        const bool rz =
            detail::select_mode(o.mode, n, o.maxdim, n ? 2.0 * double(g.m) / n : 0.0, why) == Engine::RedZeD;
        u64 edges = 0;
        Result r;
        if (rz) {
            r = redzed_result(redzed_graph(g, o.maxdim, o.threshold, &edges), o.maxdim, "sparse-redzed", why,
                              o.threshold, edges);
        } else {
            tt_barcode* b = nullptr;
            check(tt_persistence_graph_h(c, g.row_ptr.data(), g.col_idx.data(), g.weights.data(), g.n, o.maxdim,
                                         o.threshold, &b),
                  c);
            r = to_result(b, o.maxdim);
            r.stats.method = "sparse";
            r.stats.mode_reason = why;
        }
        r.stats.seconds_graph = sg;
        r.stats.seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        r.stats.peak_rss_mb = peak_rss_mb();
        return r;
    }
    if (dense || o.graph == Options::Graph::Knn) {
        std::string why;
        if (dense && detail::select_mode(o.mode, n, o.maxdim, INFINITY, why) == Engine::RedZeD) {
            for (u64 i = 0; i < u64(n) * dim; ++i)
                if (!std::isfinite(points[i])) throw std::invalid_argument("persistence: non-finite coordinate");
            // the reference relabels the points in k-d tree order first (the
            // diagram does not depend on labels; RedZeD's rows stay local)
            const PointCloud cloud{points, n, dim, Metric::minkowski(p)};
            std::vector<f32> y(u64(n) * dim);
            {
                const KdTree t(cloud);
                for (u32 i = 0; i < n; ++i) std::copy_n(points + u64(t.perm[i]) * dim, dim, y.data() + u64(i) * dim);
            }
            u64 edges = 0;
            f32 thr = INFINITY;
            rips::Barcode b = redzed_dense(y.data(), n, dim, cloud.metric, o.maxdim, INFINITY, &edges, &thr);
            Result r = redzed_result(std::move(b), o.maxdim, "dense-redzed", why, thr, edges);
            r.stats.seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            r.stats.peak_rss_mb = peak_rss_mb();
            return r;
        }
        if (o.graph == Options::Graph::Knn && o.maxdim > 0) {
            const auto tg = std::chrono::steady_clock::now();
            const PointCloud cloud{points, n, dim, Metric::minkowski(p)};
            const CsrGraph g = knn_graph_exact(cloud, o.k);
            const double sg = std::chrono::duration<double>(std::chrono::steady_clock::now() - tg).count();
            if (detail::select_mode(o.mode, n, o.maxdim, n ? 2.0 * double(g.m) / n : 0.0, why) == Engine::RedZeD) {
                u64 edges = 0;
                rips::Barcode b = redzed_graph(g, o.maxdim, o.threshold, &edges);
                Result r = redzed_result(std::move(b), o.maxdim, "sparse-redzed", why, o.threshold, edges);
                r.stats.seconds_graph = sg;
                r.stats.seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
                r.stats.peak_rss_mb = peak_rss_mb();
                return r;
            }
        }
    }
    tt_barcode* b = nullptr;
    check(tt_persistence_h(c, points, n, dim, kind, p, o.maxdim, o.threshold, o.graph == Options::Graph::Knn ? 1 : 0,
                           o.k, &b),
          c);
    Result r = to_result(b, o.maxdim);
    r.stats.seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    r.stats.peak_rss_mb = peak_rss_mb();
    return r;
}

// tops::persistence(const CsrGraph&, maxdim, threshold, threads, mode)
// (turbotops.hpp:179-207). threads and mode never change the diagram.
inline Result persistence(const CsrGraph& g, u32 maxdim, f32 threshold = INFINITY, u32 threads = 0,
                          Mode mode = Mode::Auto) {
    (void)threads;
    const auto t0 = std::chrono::steady_clock::now();
    tt_ctx* c = ctx();
    detail::validate_options(threshold, 1);
    if (!g.valid()) throw std::invalid_argument("persistence: CsrGraph invariant violated (see CsrGraph::valid)");
    std::string why;
    if (detail::select_mode(mode, g.n, maxdim, g.n ? 2.0 * double(g.m) / g.n : 0.0, why) == Engine::RedZeD) {
        u64 edges = 0;
        rips::Barcode b = redzed_graph(g, maxdim, threshold, &edges);
        Result r = redzed_result(std::move(b), maxdim, "sparse-redzed", why, threshold, edges);
        r.stats.seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        r.stats.peak_rss_mb = peak_rss_mb();
        return r;
    }
    tt_barcode* b = nullptr;
    check(tt_persistence_graph_h(c, g.row_ptr.data(), g.col_idx.data(), g.weights.data(), g.n, maxdim, threshold,
                                 &b),
          c);
    Result r = to_result(b, maxdim);
    r.stats.method = "sparse";
    r.stats.seconds_total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    r.stats.peak_rss_mb = peak_rss_mb();
    return r;
}

// knn_graph(c, knn_lists_exact(c, k)) (graph.hpp:211-225, :286-304).
inline CsrGraph knn_graph_exact(const PointCloud& pc, u32 k) {
    tt_ctx* c = ctx();
    CsrGraph g;
    g.n = pc.n;
    g.row_ptr.assign(u64(pc.n) + 1, 0);
    const u64 cap = 2ull * pc.n * (pc.n ? std::min<u32>(k, pc.n - 1) : 0);
    g.col_idx.resize(cap);
    g.weights.resize(cap);
    u64 nnz = 0;
    check(tt_knn_graph_h(c, pc.x, pc.n, pc.dim, int(pc.metric.kind), pc.metric.p, k, g.row_ptr.data(),
                         g.col_idx.data(), g.weights.data(), cap, &nnz),
          c);
    g.col_idx.resize(nnz);
    g.weights.resize(nnz);
    g.m = nnz / 2;
    return g;
}

// radius_graph (graph.hpp:170-201): the pairs with d <= tau.
inline CsrGraph radius_graph(const PointCloud& pc, f32 tau) {
    tt_ctx* c = ctx();
    CsrGraph g;
    g.n = pc.n;
    g.row_ptr.assign(u64(pc.n) + 1, 0);
    u64 nnz = 0;
    int st = tt_radius_graph_h(c, pc.x, pc.n, pc.dim, int(pc.metric.kind), pc.metric.p, tau, g.row_ptr.data(),
                               nullptr, nullptr, 0, &nnz);
    if (st == TT_ERR_LENGTH) {   // sized by the first call
        g.col_idx.resize(nnz);
        g.weights.resize(nnz);
        st = tt_radius_graph_h(c, pc.x, pc.n, pc.dim, int(pc.metric.kind), pc.metric.p, tau, g.row_ptr.data(),
                               g.col_idx.data(), g.weights.data(), nnz, &nnz);
    }
    check(st, c);
    g.m = nnz / 2;
    return g;
}

// Whole diagrams of many dense full-Rips clouds (the reference runs
// persistence(points, n, dim, Options) once per cloud; for maxdim 1 its mode
// auto takes RedZeD, turbotops.hpp:121-162, :230-259): the batched GPU front
// end computes every cloud's distance matrix, enclosing radius and sorted
// edge list in one graph launch (tt_batch_*), then the reference's RedZeD
// engine reduces the clouds on `threads` host threads (0: all), each fed with
// its cloud's matrix and edge list. Each cloud is relabelled in k-d tree order
// first, as the reference does. Other option sets run cloud by cloud through
// persistence() above. clouds[q] points at sizes[q] x dim floats.
struct BatchTiming {
    double front_s = 0, copy_s = 0, reduce_s = 0;
};
inline std::vector<Result> persistence_batch(const std::vector<const f32*>& clouds, const std::vector<u32>& sizes,
                                             u32 dim, const Options& o, u32 threads = 0,
                                             BatchTiming* timing = nullptr, bool device_predicate = true) {
    using clk = std::chrono::steady_clock;
    auto secs = [](clk::time_point a) { return std::chrono::duration<double>(clk::now() - a).count(); };
    const size_t count = clouds.size();
    std::vector<Result> out(count);
    if (clouds.size() != sizes.size()) throw std::invalid_argument("persistence_batch: clouds and sizes differ");
    tt_ctx* c = ctx();
    int kind = 0;
    float p = 2.0f;
    check(tt_metric_parse(o.metric.c_str(), &kind, &p), nullptr);
    std::string why;
    const bool batched = count && o.graph == Options::Graph::Full && std::isinf(o.threshold) && o.maxdim == 1 &&
                         detail::select_mode(o.mode, 2048, 1, INFINITY, why) == Engine::RedZeD;
    if (!batched) {
        for (size_t q = 0; q < count; ++q) out[q] = gb300::persistence(clouds[q], sizes[q], dim, o);
        return out;
    }
    const Metric metric = Metric::minkowski(p);
    // points, relabelled per cloud in k-d tree order, back to back
    u64 total = 0;
    for (u32 s : sizes) total += s;
    std::vector<f32> pts(total * dim);
    {
        u64 at = 0;
        for (size_t q = 0; q < count; ++q) {
            const u32 n = sizes[q];
            for (u64 i = 0; i < u64(n) * dim; ++i)
                if (!std::isfinite(clouds[q][i])) throw std::invalid_argument("persistence: non-finite coordinate");
            const PointCloud cloud{clouds[q], n, dim, metric};
            const KdTree t(cloud);
            for (u32 i = 0; i < n; ++i) std::copy_n(clouds[q] + u64(t.perm[i]) * dim, dim, pts.data() + (at + i) * dim);
            at += n;
        }
    }
    // make_dense's budget, cloud by cloud (rips.hpp:383-416)
    const u64 budget = o.memory_budget ? o.memory_budget : default_memory_budget();
    for (u32 s : sizes)
        if (rips::dense_bytes(s, false) > budget)
            throw std::length_error("rips: the dense distance matrix exceeds the memory budget; use a finite "
                                    "threshold or a sparse graph");
    auto t0 = clk::now();
    tt_batch* b = nullptr;
    check(tt_batch_create(c, sizes.data(), u32(count), dim, kind, p, 1, &b), c);
    struct Destroy {
        tt_batch* b;
        ~Destroy() { tt_batch_destroy(b); }
    } guard{b};
    check(tt_copy_async(c, tt_batch_points(b), pts.data(), sizeof(f32) * pts.size()), c);
    check(tt_ctx_synchronize(c), c);
    check(tt_batch_run(b, 1), c);
    tt_batch_out bo;
    check(tt_batch_result(b, &bo), c);
    if (timing) timing->front_s = secs(t0);
    t0 = clk::now();
    std::vector<f32> radius(count);
    std::vector<u64> eoff(count + 1);
    check(tt_copy_async(c, radius.data(), bo.radius_dev, 4 * count), c);
    check(tt_copy_async(c, eoff.data(), bo.edge_offset_dev, 8 * (count + 1)), c);
    check(tt_ctx_synchronize(c), c);
    std::vector<rips::DenseComplex> cx(count);
    std::vector<redzed::detail::EdgeList> el(count);
    std::vector<std::vector<uint64_t>> left(device_predicate ? count : 0);
    {
        u64 moff = 0;
        for (size_t q = 0; q < count; ++q) {
            const u32 n = sizes[q];
            if (device_predicate) {   // the leftover-coface predicate of every edge, on the device
                left[q].resize(size_t(n) * ((n + 63) / 64));
                check(tt_redzed_leftover_h(c, bo.mats_dev + moff, n, radius[q], left[q].data()), c);
            }
            cx[q].n = n;
            cx[q].full = true;
            cx[q].threshold = radius[q];
            cx[q].mat.resize(u64(n) * n);
            check(tt_copy_async(c, cx[q].mat.data(), bo.mats_dev + moff, 4 * u64(n) * n), c);
            moff += u64(n) * n;
            const u64 m = eoff[q + 1] - eoff[q];
            el[q].count = m;
            el[q].diam.resize(m);
            el[q].verts.resize(2 * m);
            if (m) {
                check(tt_copy_async(c, el[q].diam.data(), bo.diam_dev + eoff[q], 4 * m), c);
                check(tt_copy_async(c, el[q].verts.data(), bo.verts_dev + 2 * eoff[q], 8 * m), c);
            }
        }
        check(tt_ctx_synchronize(c), c);
    }
    if (timing) timing->copy_s = secs(t0);
    t0 = clk::now();
    // the clouds' reductions, largest first, on the host threads
    std::vector<size_t> order(count);
    for (size_t q = 0; q < count; ++q) order[q] = q;
    std::sort(order.begin(), order.end(), [&](size_t a, size_t bb) { return sizes[a] > sizes[bb]; });
    std::atomic<size_t> next{0};
    std::vector<std::string> errs;
    std::mutex emu;
    const u32 nt = std::max<u32>(1, std::min<u32>(threads ? threads : std::thread::hardware_concurrency(),
                                                  u32(count)));
    auto work = [&] {
        for (size_t k; (k = next.fetch_add(1)) < count;) {
            const size_t q = order[k];
            try {
                const auto tq = clk::now();
                GpuEdgesDense geo(cx[q], &el[q], device_predicate ? &left[q] : nullptr);
                u64 edges = 0;
                Result r = redzed_result(redzed::detail::run(geo, 1, cx[q].threshold, &edges), 1, "dense-redzed",
                                         why, cx[q].threshold, edges);
                r.stats.seconds_total = std::chrono::duration<double>(clk::now() - tq).count();
                out[q] = std::move(r);
                std::vector<f32>().swap(cx[q].mat);
            } catch (const std::exception& e) {
                std::lock_guard<std::mutex> l(emu);
                errs.push_back(e.what());
            }
        }
    };
    std::vector<std::thread> pool;
    for (u32 t = 1; t < nt; ++t) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
    if (!errs.empty()) throw std::runtime_error(errs[0]);
    if (timing) timing->reduce_s = secs(t0);
    return out;
}

// mst::h0 (mst.hpp:25-99): the H0 bars of the complete graph, deaths above
// the threshold essential.
inline rips::Barcode mst_h0(const PointCloud& pc, f32 threshold = INFINITY) {
    tt_ctx* c = ctx();
    tt_barcode* b = nullptr;
    check(tt_persistence_h(c, pc.x, pc.n, pc.dim, int(pc.metric.kind), pc.metric.p, 0, threshold, 0, 1, &b), c);
    return to_result(b, 0).barcode;
}

}  // namespace tops::gb300

#endif  // TURBOTOPS_GB300_HPP
