// tt_pipeline.cu — tops::persistence (turbotops.hpp:179-303) on the GB300
// front end: every data-parallel stage runs on the device, the sequential
// column reduction (compute_pairs) on the host.
//
//   maxdim = 0, full graph        complete-graph MST (mst::h0)
//   full graph, threshold = inf   dense matrix -> enclosing radius -> dim0
//                                 -> compute_pairs(1) -> assemble(1)
//                                 -> compute_pairs(2)
//   otherwise                     radius graph or kNN graph -> sparse dim0
//                                 -> compute_pairs(1)
//
// Engine choice (coboundary or RedZeD) never changes a diagram
// (turbotops.hpp:19-25); this pipeline always reduces with the cohomology
// reducer and reports the method it ran.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <unistd.h>

#include "tt_internal.cuh"
#include "tt_reduce.h"

namespace tt {

void set_thread_error(const std::string& msg);

// make_dense's memory budget (rips.hpp:383-416, turbotops.hpp:215): the full
// layout when it fits, else the lower triangle, else std::length_error. The
// device always holds the full matrix; the budget only decides whether the
// reference would have refused the complex, with its message. The default
// is the reference's: half of the host's physical memory (8 GiB if unknown).
void check_dense_budget(const tt_ctx* c, u32 n) {
    u64 budget = c->memory_budget;
    if (!budget) {
        const long pages = sysconf(_SC_PHYS_PAGES), page = sysconf(_SC_PAGE_SIZE);
        const u64 m = pages > 0 && page > 0 ? u64(pages) * u64(page) : 0;
        budget = m ? m / 2 : (u64(8) << 30);
    }
    if (u64(n) * (n ? n - 1 : 0) / 2 * sizeof(f32) > budget)
        throw Error(TT_ERR_LENGTH,
                    "rips: the dense distance matrix exceeds the memory budget; use a finite threshold or a "
                    "sparse graph");
}

namespace {

struct Result {
    std::vector<std::vector<f32>> birth, death;
    std::string method;
    f32 threshold = INFINITY;
    u64 edges = 0;
    std::vector<u64> columns, apparent, emergent;
    void ensure(u32 d) {
        if (birth.size() <= d) {
            birth.resize(d + 1);
            death.resize(d + 1);
        }
    }
    void add(u32 d, f32 b, f32 e) {
        ensure(d);
        birth[d].push_back(b);
        death[d].push_back(e);
    }
};

template <typename T>
std::vector<T> to_host(tt_ctx* c, const T* dev, u64 count) {
    std::vector<T> h(count);
    if (count) TT_CUDA(cudaMemcpyAsync(h.data(), dev, count * sizeof(T), cudaMemcpyDeviceToHost, c->stream));
    return h;
}

void sync(tt_ctx* c) { TT_CUDA(cudaStreamSynchronize(c->stream)); }

// H0 from a device dim0 result: finite bars in sorted-edge order, then one
// essential bar per component (rips.hpp:850-866).
void h0_bars(tt_ctx* c, const Dim0Out& r, Result& out) {
    const auto d = to_host(c, r.h0, r.nh0);
    sync(c);
    for (f32 v : d) out.add(0, 0.0f, v);
    for (u64 e = 0; e < r.essential; ++e) out.add(0, 0.0f, INFINITY);
}

// compute_pairs(1) over the device's dim-1 columns; returns the pivots.
std::vector<u64> reduce_dim1(tt_ctx* c, const host::HostComplex& hc, u32 maxdim, const Dim0Out& r, Result& out) {
    const auto ci = to_host(c, r.cidx, r.ncols);
    const auto cd = to_host(c, r.cd, r.ncols);
    // A graph complex with at most 8 triangles a kept edge (the benchmark's
    // 32-dimensional kNN graph: 0.77) is reduced through the boundary matrix
    // of its triangles: the same pairs and bars in the same order, without
    // cancelling the whole coboundary of every essential edge.
    const bool boundary = !hc.mat && maxdim == 1;   // (gives up past 8 triangles a kept edge)
    std::vector<u8> emf;
    std::vector<u64> emi;
    if (!boundary) {
        emi = to_host(c, r.emi, r.ncols);
        emf = to_host(c, r.emf, r.ncols);
    }
    sync(c);
    std::vector<host::Entry> cols(r.ncols);
    for (u64 i = 0; i < r.ncols; ++i) cols[i] = host::Entry{ci[i], cd[i]};
    std::vector<u64> piv;
    host::ReduceStats st;
    bool gave_up = false;
    host::Bars b;
    if (boundary) b = host::graph_pairs_dim1(hc, cols, st, &gave_up, 0, 8 * r.m);
    if (!boundary || gave_up) {   // (too many triangles, or fill-in past the cap)
        if (gave_up) {
            emi = to_host(c, r.emi, r.ncols);
            emf = to_host(c, r.emf, r.ncols);
            sync(c);
            st = host::ReduceStats{};
        }
        b = host::compute_pairs(hc, 1, maxdim, cols, emi.data(), emf.data(), piv, st);
    }
    for (u64 i = 0; i < b.birth.size(); ++i) out.add(1, b.birth[i], b.death[i]);
    out.columns.push_back(st.columns);
    out.emergent.push_back(st.emergent);
    return piv;
}

// Dimensions 2 .. maxdim on the host, for any complex: assemble(dim)
// (rips.hpp:981-1023) from every simplex of dimension dim (dimension 1: the
// kept edges dim0 sorted on the device), then compute_pairs(dim + 1), as the
// reference's Reducer::run (:1025-1031) alternates them. `piv` are the
// dimension-1 pivots.
void higher_dims(tt_ctx* c, const host::HostComplex& hc, const Dim0Out& r, std::vector<u64> piv, u32 maxdim,
                 Result& out) {
    const auto keys = to_host(c, r.keys, r.m);
    std::vector<u64> eidx;
    if (r.eidx) eidx = to_host(c, r.eidx, r.m);
    sync(c);
    std::vector<host::Entry> simp(r.m);
    for (u64 i = 0; i < r.m; ++i)
        simp[i] = r.eidx ? host::Entry{eidx[u32(keys[i])], bitsf(u32(keys[i] >> 32))}
                         : host::Entry{kIdxMask - (keys[i] & kIdxMask), bitsf(u32(keys[i] >> kIdxBits))};
    for (u32 dim = 1; dim < maxdim; ++dim) {
        std::vector<host::Entry> next;
        u64 napp = 0;
        std::sort(piv.begin(), piv.end());
        const std::vector<host::Entry> cols =
            host::assemble(hc, dim, maxdim, simp, piv, dim + 1 < maxdim ? &next : nullptr, &napp);
        out.apparent.push_back(napp);
        std::vector<u64> piv2;
        host::ReduceStats st;
        const host::Bars b = host::compute_pairs(hc, dim + 1, maxdim, cols, nullptr, nullptr, piv2, st);
        for (u64 i = 0; i < b.birth.size(); ++i) out.add(dim + 1, b.birth[i], b.death[i]);
        out.columns.push_back(st.columns);
        out.emergent.push_back(st.emergent);
        piv.swap(piv2);
        simp.swap(next);
    }
}

// Sparse front end on a device CSR graph (symmetric, rows sorted): dim0 on
// the device, H0 bars, then compute_pairs(1) on the host over the host copy
// of the graph (the caller's, or copied back here).
void sparse_tail(tt_ctx* c, u64* rp, u32* gci, f32* gw, const u64* hrp_in, const u32* hci_in, const f32* hw_in, u32 n,
                 u64 nnz, f32 thr, u32 maxdim, Result& out) {
    Complex cx{nullptr, rp, gci, gw, n, thr};
    Dim0Out r;
    dim0(c, cx, maxdim, r);
    out.edges = r.m;
    h0_bars(c, r, out);
    if (maxdim == 0) return;
    out.apparent.push_back(r.m - (n - r.essential) - r.ncols);
    std::vector<u64> hrp;
    std::vector<u32> hci;
    std::vector<f32> hw;
    if (!hrp_in) {
        hrp = to_host(c, rp, u64(n) + 1);
        hci = to_host(c, gci, nnz);
        hw = to_host(c, gw, nnz);
        sync(c);
    }
    host::HostComplex hc{nullptr, hrp_in ? hrp_in : hrp.data(), hci_in ? hci_in : hci.data(),
                         hw_in ? hw_in : hw.data(), n, thr};
    std::vector<u64> piv = reduce_dim1(c, hc, maxdim, r, out);
    if (maxdim >= 2) higher_dims(c, hc, r, std::move(piv), maxdim, out);
}

void check_points(const f32* x, u32 n, u32 dim) {
    for (u64 i = 0; i < u64(n) * dim; ++i)
        if (!std::isfinite(x[i])) invalid("persistence: non-finite coordinate");
}

void persistence_points(tt_ctx* c, const f32* x_h, u32 n, u32 dim, int kind, f32 p, u32 maxdim, f32 thr, int knn,
                        u32 k, Result& out) {
    if (std::isnan(thr) || thr < 0.0f) invalid("persistence: threshold must be non-negative or +inf");
    if (knn && k == 0) invalid("persistence: k must be >= 1");
    if (maxdim + 2 > 32) invalid("rips: maxdim must be <= 30");
    check_points(x_h, n, dim);
    out.ensure(maxdim);
    f32* x = c->arena.get<f32>(S_PTS, u64(n) * dim + 1);
    if (n) TT_CUDA(cudaMemcpyAsync(x, x_h, sizeof(f32) * n * dim, cudaMemcpyHostToDevice, c->stream));

    if (!knn && maxdim == 0) {   // mst::h0 (mst.hpp:25-99)
        out.method = "mst";
        out.threshold = thr;
        out.edges = n ? n - 1 : 0;
        if (n == 0) return;
        f32* deaths = c->arena.get<f32>(S_MISC0, n);
        mst_deaths(c, x, n, dim, kind, p, deaths);
        const auto d = to_host(c, deaths, n - 1);
        sync(c);
        u64 essential = 1;
        for (f32 v : d) {
            if (v > thr) ++essential;
            else if (v > 0.0f) out.add(0, 0.0f, v);
        }
        for (u64 e = 0; e < essential; ++e) out.add(0, 0.0f, INFINITY);
        return;
    }
    if (!knn && std::isinf(thr)) {   // dense full Rips cut at the enclosing radius
        check_dense_budget(c, n);
        out.method = "dense";
        f32* mat = c->arena.get<f32>(S_MAT, u64(n) * n + 1);
        u32* rowmax = c->arena.get<u32>(S_ROWMAX, u64(n) + 1);
        dense_matrix(c, x, n, dim, kind, p, mat, rowmax);
        f32 t = INFINITY;
        if (n) {
            min_bits(c, rowmax, n, rowmax + n);
            u32 b = 0;
            TT_CUDA(cudaMemcpyAsync(&b, rowmax + n, 4, cudaMemcpyDeviceToHost, c->stream));
            sync(c);
            t = bitsf(b);
        }
        out.threshold = t;
        if (n == 0) return;
        Complex cx{mat, nullptr, nullptr, nullptr, n, t};
        Dim0Out r;
        dim0(c, cx, maxdim, r);
        out.edges = r.m;
        h0_bars(c, r, out);
        if (maxdim == 0) return;
        out.apparent.push_back(r.m - (n - r.essential) - r.ncols);
        const auto hm = to_host(c, mat, u64(n) * n);
        sync(c);
        host::HostComplex hc{hm.data(), nullptr, nullptr, nullptr, n, t};
        std::vector<u64> piv = reduce_dim1(c, hc, maxdim, r, out);
        if (maxdim < 2) return;
        // the device assembles dimension 2 (C(n, 3) < 2^33, n <= 3740);
        // higher dimensions, or larger clouds, go through the host assemble
        if (maxdim > 2 || n > 3740) {
            higher_dims(c, hc, r, std::move(piv), maxdim, out);
            return;
        }
        u64* pd = c->arena.get<u64>(S_PIV, piv.size() + 1);
        if (!piv.empty())
            TT_CUDA(cudaMemcpyAsync(pd, piv.data(), 8 * piv.size(), cudaMemcpyHostToDevice, c->stream));
        u64* c2i = nullptr;
        f32* c2d = nullptr;
        u64 napp = 0;
        const u64 nc2 = assemble2(c, cx, r.keys, r.m, pd, piv.size(), &c2i, &c2d, &napp);
        out.apparent.push_back(napp);
        const auto ci = to_host(c, c2i, nc2);
        const auto cd = to_host(c, c2d, nc2);
        sync(c);
        std::vector<host::Entry> cols(nc2);
        for (u64 i = 0; i < nc2; ++i) cols[i] = host::Entry{ci[i], cd[i]};
        std::vector<u64> piv2;
        host::ReduceStats st;
        const host::Bars b = host::compute_pairs(hc, 2, maxdim, cols, nullptr, nullptr, piv2, st);
        for (u64 i = 0; i < b.birth.size(); ++i) out.add(2, b.birth[i], b.death[i]);
        out.columns.push_back(st.columns);
        out.emergent.push_back(st.emergent);
        return;
    }

    // graph path: radius graph (finite threshold) or the kNN graph
    out.method = "sparse";
    out.threshold = thr;
    u64* rp = c->arena.get<u64>(S_GRAPH_RP, u64(n) + 1);
    u32* ci = nullptr;
    f32* w = nullptr;
    u64 nnz = 0;
    if (knn) nnz = knn_graph(c, x, n, dim, kind, p, nullptr, n ? std::min<u32>(k, n - 1) : 0, rp, &ci, &w);
    else nnz = radius_graph(c, x, n, dim, kind, p, thr, rp, &ci, &w);
    // the kNN graph has its own slots; the radius graph's (S_OUT*) are
    // moved out of the way of the later stages
    u32* gci = ci;
    f32* gw = w;
    if (!knn) {
        gci = c->arena.get<u32>(S_GRAPH_TMP, nnz + 1);
        gw = c->arena.get<f32>(S_KNN_D, nnz + 1);
        if (nnz) {
            TT_CUDA(cudaMemcpyAsync(gci, ci, 4 * nnz, cudaMemcpyDeviceToDevice, c->stream));
            TT_CUDA(cudaMemcpyAsync(gw, w, 4 * nnz, cudaMemcpyDeviceToDevice, c->stream));
        }
    }
    if (n == 0) return;
    sparse_tail(c, rp, gci, gw, nullptr, nullptr, nullptr, n, nnz, thr, maxdim, out);
}

// tops::persistence(const CsrGraph&, maxdim, threshold) (turbotops.hpp:179-207):
// the caller's graph, checked as CsrGraph::valid() (core.hpp:137-148) does,
// uploaded, then the sparse front end.
void persistence_graph(tt_ctx* c, const u64* rp_h, const u32* ci_h, const f32* w_h, u32 n, u32 maxdim, f32 thr,
                       Result& out) {
    if (std::isnan(thr) || thr < 0.0f) invalid("persistence: threshold must be non-negative or +inf");
    if (maxdim + 2 > 32) invalid("rips: maxdim must be <= 30");
    if (!rp_h) invalid("gb300: null row_ptr");
    const u64 nnz = rp_h[n];
    bool ok = rp_h[0] == 0 && nnz % 2 == 0 && (!nnz || (ci_h && w_h));
    for (u32 v = 0; ok && v < n; ++v) {
        const u64 b = rp_h[v], e = rp_h[v + 1];
        if (e < b || e > nnz) {
            ok = false;
            break;
        }
        for (u64 t = b; t < e; ++t) {
            const u32 u = ci_h[t];
            if (u >= n || u == v || (t > b && ci_h[t - 1] >= u)) {
                ok = false;
                break;
            }
            // weight(u, v): binary search of v in row u (core.hpp:104-109)
            const u64 ub = rp_h[u], ue = rp_h[u + 1];
            if (ue < ub || ue > nnz) {
                ok = false;
                break;
            }
            const u32* it = std::lower_bound(ci_h + ub, ci_h + ue, v);
            const f32 wuv = (it != ci_h + ue && *it == v) ? w_h[it - ci_h] : INFINITY;
            if (wuv != w_h[t]) {
                ok = false;
                break;
            }
        }
    }
    if (!ok) invalid("persistence: CsrGraph invariant violated (see CsrGraph::valid)");
    out.ensure(maxdim);
    out.method = "sparse";
    out.threshold = thr;
    if (n == 0) return;
    u64* rp = c->arena.get<u64>(S_GRAPH_RP, u64(n) + 1);
    u32* gci = c->arena.get<u32>(S_GRAPH_TMP, nnz + 1);
    f32* gw = c->arena.get<f32>(S_KNN_D, nnz + 1);
    TT_CUDA(cudaMemcpyAsync(rp, rp_h, 8 * (u64(n) + 1), cudaMemcpyHostToDevice, c->stream));
    if (nnz) {
        TT_CUDA(cudaMemcpyAsync(gci, ci_h, 4 * nnz, cudaMemcpyHostToDevice, c->stream));
        TT_CUDA(cudaMemcpyAsync(gw, w_h, 4 * nnz, cudaMemcpyHostToDevice, c->stream));
    }
    sparse_tail(c, rp, gci, gw, rp_h, ci_h, w_h, n, nnz, thr, maxdim, out);
}

}  // namespace
}  // namespace tt

using namespace tt;

namespace {
template <typename F>
int guarded(tt_ctx* c, F&& f) {
    try {
        if (!c) throw Error(TT_ERR_INVALID, "gb300: null context");
        TT_CUDA(cudaSetDevice(c->device));
        f();
        return TT_OK;
    } catch (const Error& e) {
        c ? (void)(c->last_error = e.what()) : set_thread_error(e.what());
        return e.status;
    } catch (const std::exception& e) {
        c ? (void)(c->last_error = e.what()) : set_thread_error(e.what());
        return TT_ERR_INTERNAL;
    }
}

tt_barcode* pack(const Result& r) {
    auto* b = static_cast<tt_barcode*>(std::calloc(1, sizeof(tt_barcode)));
    b->ndims = u32(r.birth.size());
    u64 total = 0;
    for (auto& v : r.birth) total += v.size();
    b->total = total;
    b->count = static_cast<uint64_t*>(std::calloc(b->ndims + 1, sizeof(uint64_t)));
    b->birth = static_cast<float*>(std::malloc(sizeof(float) * (total + 1)));
    b->death = static_cast<float*>(std::malloc(sizeof(float) * (total + 1)));
    u64 o = 0;
    for (u32 d = 0; d < b->ndims; ++d) {
        b->count[d] = r.birth[d].size();
        for (u64 i = 0; i < r.birth[d].size(); ++i, ++o) {
            b->birth[o] = r.birth[d][i];
            b->death[o] = r.death[d][i];
        }
    }
    std::snprintf(b->method, sizeof(b->method), "%s", r.method.c_str());
    b->threshold = r.threshold;
    b->edges = r.edges;
    for (u64 i = 0; i < r.columns.size() && i < 32; ++i) b->columns[i] = r.columns[i];
    for (u64 i = 0; i < r.apparent.size() && i < 32; ++i) b->apparent[i] = r.apparent[i];
    for (u64 i = 0; i < r.emergent.size() && i < 32; ++i) b->emergent[i] = r.emergent[i];
    return b;
}
}  // namespace

extern "C" int tt_persistence_h(tt_ctx* c, const float* x_h, uint32_t n, uint32_t dim, int kind, float p,
                                uint32_t maxdim, float threshold, int knn, uint32_t k, tt_barcode** out) {
    return guarded(c, [&] {
        if (!out) invalid("gb300: null output");
        *out = nullptr;
        if (kind < TT_METRIC_L1 || kind > TT_METRIC_LP) invalid("metric: unknown kind");
        if (kind == TT_METRIC_LP && !(p >= 1.0f)) invalid("metric: p must be in [1, inf]");
        Result r;
        persistence_points(c, x_h, n, dim, kind, p, maxdim, threshold, knn, k, r);
        *out = pack(r);
    });
}

extern "C" int tt_persistence_graph_h(tt_ctx* c, const uint64_t* row_ptr_h, const uint32_t* col_h,
                                      const float* weight_h, uint32_t n, uint32_t maxdim, float threshold,
                                      tt_barcode** out) {
    return guarded(c, [&] {
        if (!out) invalid("gb300: null output");
        *out = nullptr;
        Result r;
        persistence_graph(c, row_ptr_h, col_h, weight_h, n, maxdim, threshold, r);
        *out = pack(r);
    });
}

extern "C" void tt_barcode_free(tt_barcode* b) {
    if (!b) return;
    std::free(b->count);
    std::free(b->birth);
    std::free(b->death);
    std::free(b);
}
