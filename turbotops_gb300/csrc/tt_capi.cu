// tt_capi.cu — the C-ABI (include/turbotops_gb300.h): argument checks with the
// reference's messages, exception -> status mapping, host-buffer entry points.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>

#include "tt_internal.cuh"

using namespace tt;

namespace {

thread_local std::string g_error;   // errors of calls without a context

// A call that checked its points asynchronously (check_finite_async) and
// failed before reading the result reports the non-finite coordinate, which
// the reference detects before anything else.
bool nonfinite_pending(tt_ctx* c) {
    if (!c || !c->fin_pending) return false;
    c->fin_pending = false;
    return cudaEventSynchronize(c->fin_ev) == cudaSuccess && *c->fin_host != 0;
}

template <typename F>
int guard(tt_ctx* c, F&& f) {
    try {
        if (!c) throw Error(TT_ERR_INVALID, "gb300: null context");
        c->fin_pending = false;
        TT_CUDA(cudaSetDevice(c->device));
        f();
        return TT_OK;
    } catch (const Error& e) {
        if (nonfinite_pending(c)) {
            c->last_error = "persistence: non-finite coordinate";
            return TT_ERR_INVALID;
        }
        (c ? c->last_error : g_error) = e.what();
        return e.status;
    } catch (const std::exception& e) {
        if (nonfinite_pending(c)) {
            c->last_error = "persistence: non-finite coordinate";
            return TT_ERR_INVALID;
        }
        (c ? c->last_error : g_error) = e.what();
        return TT_ERR_INTERNAL;
    }
}

// Any non-finite coordinate among count floats of a device buffer? (One
// pass on the device instead of a scalar host loop over the caller's array.)
__global__ void k_nonfinite(const f32* __restrict__ x, u64 count, u32* __restrict__ flag) {
    u32 bad = 0;
    for (u64 i = u64(blockIdx.x) * blockDim.x + threadIdx.x; i < count; i += u64(gridDim.x) * blockDim.x)
        bad |= (__float_as_uint(x[i]) & 0x7f800000u) == 0x7f800000u;
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1u);
}

// The same test storing 1 into a flag when some coordinate is not finite
// (every writer stores the same value), four floats a load when aligned.
__global__ void k_nonfinite_store(const f32* __restrict__ x, u64 count, unsigned* flag) {
    u32 bad = 0;
    const u64 stride = u64(gridDim.x) * blockDim.x;
    const u64 t0 = u64(blockIdx.x) * blockDim.x + threadIdx.x;
    u64 head = 0;   // floats before the first 16-byte boundary
    if ((reinterpret_cast<uintptr_t>(x) & 15) != 0) head = min(count, u64((16 - (reinterpret_cast<uintptr_t>(x) & 15)) / 4));
    for (u64 i = t0; i < head; i += stride) bad |= (__float_as_uint(x[i]) & 0x7f800000u) == 0x7f800000u;
    const float4* v = reinterpret_cast<const float4*>(x + head);
    const u64 nv = (count - head) / 4;
    for (u64 i = t0; i < nv; i += stride) {
        const float4 f = __ldg(v + i);
        bad |= ((__float_as_uint(f.x) & 0x7f800000u) == 0x7f800000u) | ((__float_as_uint(f.y) & 0x7f800000u) == 0x7f800000u) |
               ((__float_as_uint(f.z) & 0x7f800000u) == 0x7f800000u) | ((__float_as_uint(f.w) & 0x7f800000u) == 0x7f800000u);
    }
    for (u64 i = head + nv * 4 + t0; i < count; i += stride) bad |= (__float_as_uint(x[i]) & 0x7f800000u) == 0x7f800000u;
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) *reinterpret_cast<volatile unsigned*>(flag) = 1u;
}

void check_finite_dev(tt_ctx* c, const f32* x, u64 count) {
    if (!count) return;
    u32* flag = c->arena.get<u32>(S_MISC2, 4);
    TT_CUDA(cudaMemsetAsync(flag, 0, sizeof(u32), c->stream));
    const u32 grid = u32(std::min<u64>((count + 255) / 256, 4ull * u64(c->sms)));
    k_nonfinite<<<grid, 256, 0, c->stream>>>(x, count, flag);
    TT_LAUNCH("k_nonfinite");
    ++c->launches;
    u32 h = 0;
    TT_CUDA(cudaMemcpyAsync(&h, flag, sizeof(u32), cudaMemcpyDeviceToHost, c->stream));
    TT_CUDA(cudaStreamSynchronize(c->stream));
    if (h) invalid("persistence: non-finite coordinate");
}

}  // namespace

namespace tt {
// The same check without the round trip: the flag goes to page-locked memory
// and settle_finite reads it once the next stages are enqueued, before any
// kernel indexes memory by a value derived from the points (the kNN kernels
// only compare distances: a NaN never enters a list).
void check_finite_async(tt_ctx* c, const f32* x, u64 count) {
    c->fin_pending = false;
    if (!count) return;
    if (!c->fin_host) {
        TT_CUDA(cudaHostAlloc(&c->fin_host, sizeof(unsigned), cudaHostAllocMapped));
        TT_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void**>(&c->fin_dev), c->fin_host, 0));
    }
    if (!c->fin_ev) TT_CUDA(cudaEventCreateWithFlags(&c->fin_ev, cudaEventDisableTiming));
    // the flag lives in mapped page-locked memory: the kernel stores into it
    // directly, so nothing but the kernel itself sits in the stream (the
    // previous call's kernel has completed: its event was waited for)
    *reinterpret_cast<volatile unsigned*>(c->fin_host) = 0u;
    const u32 grid = u32(std::min<u64>((count + 1023) / 1024, 4ull * u64(c->sms)));
    k_nonfinite_store<<<grid, 256, 0, c->stream>>>(x, count, c->fin_dev);
    TT_LAUNCH("k_nonfinite");
    ++c->launches;
    TT_CUDA(cudaEventRecord(c->fin_ev, c->stream));
    c->fin_pending = true;
}

void settle_finite(tt_ctx* c) {
    if (!c->fin_pending) return;
    c->fin_pending = false;
    TT_CUDA(cudaEventSynchronize(c->fin_ev));
    if (*c->fin_host) invalid("persistence: non-finite coordinate");
}
}  // namespace tt

namespace {

void check_metric(int kind, float p) {
    if (kind < TT_METRIC_L1 || kind > TT_METRIC_LP) invalid("metric: unknown kind");
    if (kind == TT_METRIC_LP && !(p >= 1.0f)) invalid("metric: p must be in [1, inf]");
}

void fill_dim0(const Dim0Out& r, tt_dim0_out* out) {
    out->edges = r.m;
    out->edge_keys_dev = r.keys;
    out->apparent_dev = r.app;
    out->tree_dev = r.tree;
    out->columns = r.ncols;
    out->col_index_dev = r.cidx;
    out->col_diameter_dev = r.cd;
    out->col_cofacet_dev = r.emi;
    out->col_cofacet_app_dev = r.emf;
    out->h0_finite = r.nh0;
    out->h0_death_dev = r.h0;
    out->essential = r.essential;
}

// Is p page-locked host memory (so that copies into it are asynchronous)?
bool pinned_host(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// The context's second stream, ordered after everything enqueued on its
// main stream so far.
cudaStream_t aux_after_main(tt_ctx* c) {
    if (!c->aux) TT_CUDA(cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking));
    if (!c->aux_ev) TT_CUDA(cudaEventCreateWithFlags(&c->aux_ev, cudaEventDisableTiming));
    TT_CUDA(cudaEventRecord(c->aux_ev, c->stream));
    TT_CUDA(cudaStreamWaitEvent(c->aux, c->aux_ev, 0));
    return c->aux;
}

// knn_lists_exact -> knn_graph -> dim0 on the device. The graph is moved into
// slots that dim0 does not use, so both results stay valid together.
template <typename AfterGraph>
u64 knn_front_dev(tt_ctx* c, const f32* x, u32 n, u32 dim, int kind, f32 p, u32 k, u32 maxdim, u64** rp_out,
                  u32** ci_out, f32** w_out, Dim0Out& r, AfterGraph&& after_graph) {
    const u32 kk = n ? std::min<u32>(k, n - 1) : 0;
    u64* rp = c->arena.get<u64>(S_GRAPH_RP, u64(n) + 1);
    u32* ci = nullptr;
    f32* w = nullptr;
    const u64 nnz = knn_graph(c, x, n, dim, kind, p, nullptr, kk, rp, &ci, &w);   // its own slots: dim0 keeps them
    u32* gci = ci;
    f32* gw = w;
    after_graph(nnz, rp, gci, gw);   // before dim0: the graph is final here
    Complex cx{nullptr, rp, gci, gw, n, INFINITY};
    dim0(c, cx, maxdim, r, nnz / 2);   // symmetric, no self loops, cut at +inf: every edge kept
    *rp_out = rp;
    *ci_out = gci;
    *w_out = gw;
    return nnz;
}

}  // namespace

namespace tt {
// Error text for context-free entry points (read back by tt_last_error(NULL)).
void set_thread_error(const std::string& msg) { g_error = msg; }
}  // namespace tt

extern "C" {

const char* tt_version(void) { return "0.1.0"; }

int tt_ctx_create(int device, void* stream, tt_ctx** out) {
    if (!out) return TT_ERR_INVALID;
    *out = nullptr;
    tt_ctx* c = new tt_ctx;
    c->device = device;
    const int st = guard(c, [&] {
        cudaDeviceProp prop;
        TT_CUDA(cudaGetDeviceProperties(&prop, device));
        c->sms = prop.multiProcessorCount;
        // The stream is used as given; NULL is the legacy default stream.
        c->stream = static_cast<cudaStream_t>(stream);
    });
    if (st != TT_OK) {
        g_error = c->last_error;
        delete c;
        return st;
    }
    *out = c;
    return TT_OK;
}

void tt_ctx_destroy(tt_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    c->arena.release();
    c->pinned.release();
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    if (c->aux) {
        cudaStreamSynchronize(c->aux);
        cudaStreamDestroy(c->aux);
    }
    if (c->aux_ev) cudaEventDestroy(c->aux_ev);
    if (c->tc_host) cudaFreeHost(c->tc_host);
    if (c->fin_host) cudaFreeHost(c->fin_host);
    if (c->fin_ev) cudaEventDestroy(c->fin_ev);
    if (c->side) {
        cudaStreamSynchronize(c->side);
        cudaStreamDestroy(c->side);
    }
    for (auto e : c->side_ev)
        if (e) cudaEventDestroy(e);
    delete c;
}

const char* tt_last_error(const tt_ctx* c) { return c ? c->last_error.c_str() : g_error.c_str(); }

uint64_t tt_ctx_launches(const tt_ctx* c) { return c ? c->launches : 0; }

int tt_ctx_synchronize(tt_ctx* c) {
    return guard(c, [&] { TT_CUDA(cudaStreamSynchronize(c->stream)); });
}

int tt_ctx_set_knn_mode(tt_ctx* c, int mode) {
    return guard(c, [&] {
        if (mode < 0 || mode > 2) invalid("gb300: knn mode must be 0, 1 or 2");
        c->knn_mode = mode;
    });
}

int tt_ctx_set_memory_budget(tt_ctx* c, uint64_t bytes) {
    return guard(c, [&] { c->memory_budget = bytes; });
}

uint64_t tt_ctx_filter_evals(const tt_ctx* c) { return c ? c->filter_evals : 0; }
uint64_t tt_ctx_filter_tiles(const tt_ctx* c) { return c ? c->filter_tiles : 0; }

int tt_tc_gram_check(tt_ctx* c, uint32_t products, uint64_t seed, double* max_rel) {
    return guard(c, [&] {
        if (!max_rel) invalid("gb300: null output");
        *max_rel = tc_gram_check(c, products, seed);
    });
}

int tt_selftest_wait_timeout(tt_ctx* c, uint32_t polls) {
    return guard(c, [&] { selftest_wait_timeout(c, polls); });
}

int tt_ctx_inject_alloc_failure(tt_ctx* c, uint32_t nth) {
    return guard(c, [&] { c->arena.fail_in = nth; });
}

int tt_copy_async(tt_ctx* c, void* dst, const void* src, size_t bytes) {
    return guard(c, [&] {
        if (bytes) TT_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, c->stream));
    });
}

int tt_metric_parse(const char* s, int* kind, float* p) {
    // Metric::parse / Metric::minkowski (metric.hpp:227-253)
    const std::string m = s ? s : "";
    float q = NAN;
    if (m == "l2" || m == "euclidean") q = 2.0f;
    else if (m == "l1" || m == "manhattan") q = 1.0f;
    else if (m == "linf" || m == "chebyshev") q = INFINITY;
    else if (m.rfind("lp:", 0) == 0) {
        const std::string v = m.substr(3);
        if (v == "inf") q = INFINITY;
        else {
            char* end = nullptr;
            const float t = std::strtof(v.c_str(), &end);
            if (end && *end == '\0' && !v.empty()) q = t;
            else goto unknown;
        }
    } else {
        goto unknown;
    }
    if (!(q >= 1.0f)) {
        g_error = "metric: p must be in [1, inf]";
        return TT_ERR_INVALID;
    }
    *p = q;
    *kind = q == 1.0f ? TT_METRIC_L1 : q == 2.0f ? TT_METRIC_L2 : std::isinf(q) ? TT_METRIC_LINF : TT_METRIC_LP;
    return TT_OK;
unknown:
    g_error = "metric: unknown '" + m + "' (expected l1 | l2 | linf | lp:<p>, p >= 1)";
    return TT_ERR_INVALID;
}

int tt_dense_distances(tt_ctx* c, const float* x, uint32_t n, uint32_t dim, int kind, float p, float* mat,
                       float* enclosing) {
    return guard(c, [&] {
        check_metric(kind, p);
        if (n && (!x || !mat)) invalid("gb300: null buffer");
        u32* rowmax = enclosing ? c->arena.get<u32>(S_ROWMAX, u64(n) + 1) : nullptr;
        dense_matrix(c, x, n, dim, kind, p, mat, rowmax);
        if (enclosing) {
            if (n == 0) {
                *enclosing = INFINITY;
                return;
            }
            min_bits(c, rowmax, n, rowmax + n);
            u32 b = 0;
            TT_CUDA(cudaMemcpyAsync(&b, rowmax + n, 4, cudaMemcpyDeviceToHost, c->stream));
            TT_CUDA(cudaStreamSynchronize(c->stream));
            *enclosing = bitsf(b);
        }
    });
}

int tt_dim0(tt_ctx* c, const float* mat, const uint64_t* rp, const uint32_t* ci, const float* w, uint32_t n,
            float thr, uint32_t maxdim, tt_dim0_out* out) {
    return guard(c, [&] {
        if (!out) invalid("gb300: null output");
        if (std::isnan(thr) || thr < 0.0f) invalid("persistence: threshold must be non-negative or +inf");
        if (n > 1 && !mat && !(rp && ci && w)) invalid("gb300: null complex");
        if (n > kPackedMaxN) invalid("gb300: tt_dim0's packed edge keys support n <= 131072 vertices");
        Complex cx{mat, rp, ci, w, n, thr};
        Dim0Out r;
        dim0(c, cx, maxdim, r);
        out->edges = r.m;
        out->edge_keys_dev = r.keys;
        out->apparent_dev = r.app;
        out->tree_dev = r.tree;
        out->columns = r.ncols;
        out->col_index_dev = r.cidx;
        out->col_diameter_dev = r.cd;
        out->col_cofacet_dev = r.emi;
        out->col_cofacet_app_dev = r.emf;
        out->h0_finite = r.nh0;
        out->h0_death_dev = r.h0;
        out->essential = r.essential;
    });
}

int tt_redzed_edges(tt_ctx* c, const float* mat, const uint64_t* rp, const uint32_t* ci, const float* w,
                    uint32_t n, float thr, float* diam, int32_t* verts, uint64_t cap, uint64_t* count) {
    return guard(c, [&] {
        if (std::isnan(thr) || thr < 0.0f) invalid("persistence: threshold must be non-negative or +inf");
        Complex cx{mat, rp, ci, w, n, thr};
        const u64 m = redzed_edges(c, cx, diam, verts, cap);
        if (count) *count = m;
        if (m > cap) throw Error(TT_ERR_LENGTH, "gb300: edge list exceeds the output capacity");
    });
}

int tt_assemble(tt_ctx* c, const float* mat, uint32_t n, float thr, const uint64_t* keys, uint64_t m,
                const uint64_t* piv, uint64_t npiv, uint64_t* columns, const uint64_t** cidx, const float** cd,
                uint64_t* apparent) {
    return guard(c, [&] {
        if (std::isnan(thr) || thr < 0.0f) invalid("persistence: threshold must be non-negative or +inf");
        if (!columns || !cidx || !cd) invalid("gb300: null output");
        Complex cx{mat, nullptr, nullptr, nullptr, n, thr};
        u64* ci = nullptr;
        f32* d = nullptr;
        u64 napp = 0;
        *columns = assemble2(c, cx, keys, m, piv, npiv, &ci, &d, &napp);
        *cidx = ci;
        *cd = d;
        if (apparent) *apparent = napp;
    });
}

int tt_knn(tt_ctx* c, const float* x, uint32_t n, uint32_t dim, int kind, float p, uint32_t k, uint32_t* ids,
           float* dists, uint32_t* k_out) {
    return guard(c, [&] {
        check_metric(kind, p);
        if (k == 0) invalid("persistence: k must be >= 1");
        const u32 kk = n ? std::min<u32>(k, n - 1) : 0;
        if (k_out) *k_out = kk;
        if (kk) knn_exact(c, x, n, dim, kind, p, kk, ids, dists);
    });
}

int tt_knn_graph(tt_ctx* c, const float* x, uint32_t n, uint32_t dim, int kind, float p, uint32_t k,
                 tt_csr_out* out) {
    return guard(c, [&] {
        check_metric(kind, p);
        if (k == 0) invalid("persistence: k must be >= 1");
        if (!out) invalid("gb300: null output");
        const u32 kk = n ? std::min<u32>(k, n - 1) : 0;
        u64* rp = c->arena.get<u64>(S_OUT0, u64(n) + 1);
        u32* ci = nullptr;
        f32* w = nullptr;
        // a NaN leaves a list short: the graph build reads the check first
        check_finite_async(c, x, u64(n) * dim);
        const u64 nnz = knn_graph(c, x, n, dim, kind, p, nullptr, kk, rp, &ci, &w);
        out->n = n;
        out->nnz = nnz;
        out->row_ptr_dev = rp;
        out->col_dev = ci;
        out->weight_dev = w;
    });
}

int tt_radius_graph(tt_ctx* c, const float* x, uint32_t n, uint32_t dim, int kind, float p, float tau,
                    tt_csr_out* out) {
    return guard(c, [&] {
        check_metric(kind, p);
        if (std::isnan(tau) || tau < 0.0f) invalid("persistence: threshold must be non-negative or +inf");
        if (!out) invalid("gb300: null output");
        u64* rp = c->arena.get<u64>(S_OUT0, u64(n) + 1);
        u32* ci = nullptr;
        f32* w = nullptr;
        const u64 nnz = radius_graph(c, x, n, dim, kind, p, tau, rp, &ci, &w);
        out->n = n;
        out->nnz = nnz;
        out->row_ptr_dev = rp;
        out->col_dev = ci;
        out->weight_dev = w;
    });
}

int tt_mst_deaths(tt_ctx* c, const float* x, uint32_t n, uint32_t dim, int kind, float p, float* deaths) {
    return guard(c, [&] {
        check_metric(kind, p);
        check_finite_async(c, x, u64(n) * dim);   // read before the rounds index anything by a list entry
        mst_deaths(c, x, n, dim, kind, p, deaths);
        settle_finite(c);
    });
}

int tt_knn_graph_h(tt_ctx* c, const float* x_h, uint32_t n, uint32_t dim, int kind, float p, uint32_t k,
                   uint64_t* rp_h, uint32_t* col_h, float* w_h, uint64_t cap, uint64_t* nnz_out) {
    return guard(c, [&] {
        check_metric(kind, p);
        if (k == 0) invalid("persistence: k must be >= 1");
        f32* x = c->arena.get<f32>(S_PTS, u64(n) * dim + 1);
        if (n) TT_CUDA(cudaMemcpyAsync(x, x_h, sizeof(f32) * n * dim, cudaMemcpyHostToDevice, c->stream));
        check_finite_dev(c, x, u64(n) * dim);
        const u32 kk = n ? std::min<u32>(k, n - 1) : 0;
        u64* rp = c->arena.get<u64>(S_OUT0, u64(n) + 1);
        u32* ci = nullptr;
        f32* w = nullptr;
        const u64 nnz = knn_graph(c, x, n, dim, kind, p, nullptr, kk, rp, &ci, &w);
        if (nnz_out) *nnz_out = nnz;
        if (nnz > cap) throw Error(TT_ERR_LENGTH, "gb300: graph exceeds the output capacity");
        TT_CUDA(cudaMemcpyAsync(rp_h, rp, 8 * (u64(n) + 1), cudaMemcpyDeviceToHost, c->stream));
        if (nnz) {
            TT_CUDA(cudaMemcpyAsync(col_h, ci, 4 * nnz, cudaMemcpyDeviceToHost, c->stream));
            TT_CUDA(cudaMemcpyAsync(w_h, w, 4 * nnz, cudaMemcpyDeviceToHost, c->stream));
        }
        TT_CUDA(cudaStreamSynchronize(c->stream));
    });
}

int tt_radius_graph_h(tt_ctx* c, const float* x_h, uint32_t n, uint32_t dim, int kind, float p, float tau,
                      uint64_t* rp_h, uint32_t* col_h, float* w_h, uint64_t cap, uint64_t* nnz_out) {
    return guard(c, [&] {
        check_metric(kind, p);
        if (std::isnan(tau) || tau < 0.0f) invalid("persistence: threshold must be non-negative or +inf");
        f32* x = c->arena.get<f32>(S_PTS, u64(n) * dim + 1);
        if (n) TT_CUDA(cudaMemcpyAsync(x, x_h, sizeof(f32) * n * dim, cudaMemcpyHostToDevice, c->stream));
        check_finite_dev(c, x, u64(n) * dim);
        u64* rp = c->arena.get<u64>(S_OUT0, u64(n) + 1);
        u32* ci = nullptr;
        f32* w = nullptr;
        const u64 nnz = radius_graph(c, x, n, dim, kind, p, tau, rp, &ci, &w);
        if (nnz_out) *nnz_out = nnz;
        if (nnz > cap) throw Error(TT_ERR_LENGTH, "gb300: graph exceeds the output capacity");
        TT_CUDA(cudaMemcpyAsync(rp_h, rp, 8 * (u64(n) + 1), cudaMemcpyDeviceToHost, c->stream));
        if (nnz) {
            TT_CUDA(cudaMemcpyAsync(col_h, ci, 4 * nnz, cudaMemcpyDeviceToHost, c->stream));
            TT_CUDA(cudaMemcpyAsync(w_h, w, 4 * nnz, cudaMemcpyDeviceToHost, c->stream));
        }
        TT_CUDA(cudaStreamSynchronize(c->stream));
    });
}

int tt_knn_front(tt_ctx* c, const float* x, uint32_t n, uint32_t dim, int kind, float p, uint32_t k,
                 uint32_t maxdim, tt_knn_front_out* out) {
    return guard(c, [&] {
        check_metric(kind, p);
        if (k == 0) invalid("persistence: k must be >= 1");
        if (!out) invalid("gb300: null output");
        if (n > kPackedMaxN) invalid("gb300: tt_knn_front's packed edge keys support n <= 131072 vertices");
        check_finite_async(c, x, u64(n) * dim);   // read by the graph build (a NaN leaves a list short)
        u64* rp = nullptr;
        u32* ci = nullptr;
        f32* w = nullptr;
        Dim0Out r;
        const u64 nnz = knn_front_dev(c, x, n, dim, kind, p, k, maxdim, &rp, &ci, &w, r, [](u64, u64*, u32*, f32*) {});
        out->graph.n = n;
        out->graph.nnz = nnz;
        out->graph.row_ptr_dev = rp;
        out->graph.col_dev = ci;
        out->graph.weight_dev = w;
        fill_dim0(r, &out->dim0);
    });
}

int tt_knn_front_h(tt_ctx* c, const float* x_h, uint32_t n, uint32_t dim, int kind, float p, uint32_t k,
                   uint32_t maxdim, uint64_t* rp_h, uint32_t* col_h, float* w_h, uint64_t cap, uint64_t* nnz_out,
                   float* h0_h, uint64_t* nh0, uint64_t* essential, uint64_t* col_idx_h, float* col_d_h,
                   uint64_t* col_cf_h, uint8_t* col_cf_app_h, uint64_t col_cap, uint64_t* ncols,
                   uint64_t* nedges) {
    return guard(c, [&] {
        check_metric(kind, p);
        if (k == 0) invalid("persistence: k must be >= 1");
        f32* x = c->arena.get<f32>(S_PTS, u64(n) * dim + 1);
        if (n) TT_CUDA(cudaMemcpyAsync(x, x_h, sizeof(f32) * n * dim, cudaMemcpyHostToDevice, c->stream));
        check_finite_async(c, x, u64(n) * dim);   // read in knn_graph, after the kNN is enqueued
        u64* rp = nullptr;
        u32* gci = nullptr;
        f32* gw = nullptr;
        Dim0Out r;
        // The graph is final before dim0 starts: into page-locked buffers it
        // is copied on the context's second stream while dim0 runs.
        bool early = false;
        auto copy_graph = [&](cudaStream_t s, u64 nnz, const u64* rpd, const u32* cid, const f32* wd) {
            TT_CUDA(cudaMemcpyAsync(rp_h, rpd, 8 * (u64(n) + 1), cudaMemcpyDeviceToHost, s));
            if (nnz) {
                TT_CUDA(cudaMemcpyAsync(col_h, cid, 4 * nnz, cudaMemcpyDeviceToHost, s));
                TT_CUDA(cudaMemcpyAsync(w_h, wd, 4 * nnz, cudaMemcpyDeviceToHost, s));
            }
        };
        struct AuxDrain {   // no copy outlives the call, whatever path leaves it
            tt_ctx* c;
            bool& on;
            ~AuxDrain() {
                if (on) cudaStreamSynchronize(c->aux);
            }
        } drain{c, early};
        const u64 nnz = knn_front_dev(c, x, n, dim, kind, p, k, maxdim, &rp, &gci, &gw, r,
                                      [&](u64 m, u64* rpd, u32* cid, f32* wd) {
                                          if (nnz_out) *nnz_out = m;
                                          if (m > cap)
                                              throw Error(TT_ERR_LENGTH, "gb300: graph exceeds the output capacity");
                                          if (pinned_host(rp_h) && (!m || (pinned_host(col_h) && pinned_host(w_h)))) {
                                              copy_graph(aux_after_main(c), m, rpd, cid, wd);
                                              early = true;
                                          }
                                      });
        if (!early) copy_graph(c->stream, nnz, rp, gci, gw);
        if (h0_h && r.nh0)
            TT_CUDA(cudaMemcpyAsync(h0_h, r.h0, sizeof(f32) * r.nh0, cudaMemcpyDeviceToHost, c->stream));
        if (nh0) *nh0 = r.nh0;
        if (essential) *essential = r.essential;
        if (ncols) *ncols = r.ncols;
        if (nedges) *nedges = r.m;
        if (col_idx_h && r.ncols) {
            if (r.ncols > col_cap) throw Error(TT_ERR_LENGTH, "gb300: columns exceed the output capacity");
            TT_CUDA(cudaMemcpyAsync(col_idx_h, r.cidx, 8 * r.ncols, cudaMemcpyDeviceToHost, c->stream));
            if (col_d_h) TT_CUDA(cudaMemcpyAsync(col_d_h, r.cd, 4 * r.ncols, cudaMemcpyDeviceToHost, c->stream));
            if (col_cf_h) TT_CUDA(cudaMemcpyAsync(col_cf_h, r.emi, 8 * r.ncols, cudaMemcpyDeviceToHost, c->stream));
            if (col_cf_app_h)
                TT_CUDA(cudaMemcpyAsync(col_cf_app_h, r.emf, r.ncols, cudaMemcpyDeviceToHost, c->stream));
        }
        TT_CUDA(cudaStreamSynchronize(c->stream));
        if (early) {
            early = false;
            TT_CUDA(cudaStreamSynchronize(c->aux));
        }
    });
}

int tt_dense_front_h(tt_ctx* c, const float* x_h, uint32_t n, uint32_t dim, int kind, float p, uint32_t maxdim,
                     float* thr_inout, float* mat_h, float* h0_h, uint64_t* nh0, uint64_t* essential,
                     uint64_t* col_idx_h, float* col_d_h, uint64_t* col_cf_h, uint8_t* col_cf_app_h,
                     uint64_t col_cap, uint64_t* ncols, uint64_t* nedges) {
    return guard(c, [&] {
        check_metric(kind, p);
        if (!thr_inout) invalid("gb300: null threshold");
        const float t = *thr_inout;
        if (std::isnan(t) || t < 0.0f) invalid("persistence: threshold must be non-negative or +inf");
        check_dense_budget(c, n);
        f32* x = c->arena.get<f32>(S_PTS, u64(n) * dim + 1);
        if (n) TT_CUDA(cudaMemcpyAsync(x, x_h, sizeof(f32) * n * dim, cudaMemcpyHostToDevice, c->stream));
        check_finite_dev(c, x, u64(n) * dim);
        f32* mat = c->arena.get<f32>(S_MAT, u64(n) * n + 1);
        u32* rowmax = c->arena.get<u32>(S_ROWMAX, u64(n) + 1);
        dense_matrix(c, x, n, dim, kind, p, mat, std::isinf(t) ? rowmax : nullptr);
        float thr = t;
        if (std::isinf(t)) {
            if (n == 0) {
                thr = INFINITY;
            } else {
                min_bits(c, rowmax, n, rowmax + n);
                u32 b = 0;
                TT_CUDA(cudaMemcpyAsync(&b, rowmax + n, 4, cudaMemcpyDeviceToHost, c->stream));
                TT_CUDA(cudaStreamSynchronize(c->stream));
                thr = bitsf(b);
            }
        }
        *thr_inout = thr;
        Complex cx{mat, nullptr, nullptr, nullptr, n, thr};
        Dim0Out r;
        dim0(c, cx, maxdim, r);
        if (mat_h && n)
            TT_CUDA(cudaMemcpyAsync(mat_h, mat, sizeof(f32) * n * n, cudaMemcpyDeviceToHost, c->stream));
        if (h0_h && r.nh0)
            TT_CUDA(cudaMemcpyAsync(h0_h, r.h0, sizeof(f32) * r.nh0, cudaMemcpyDeviceToHost, c->stream));
        if (col_idx_h && r.ncols) {
            if (r.ncols > col_cap) throw Error(TT_ERR_LENGTH, "gb300: columns exceed the output capacity");
            TT_CUDA(cudaMemcpyAsync(col_idx_h, r.cidx, 8 * r.ncols, cudaMemcpyDeviceToHost, c->stream));
            if (col_d_h) TT_CUDA(cudaMemcpyAsync(col_d_h, r.cd, 4 * r.ncols, cudaMemcpyDeviceToHost, c->stream));
            if (col_cf_h) TT_CUDA(cudaMemcpyAsync(col_cf_h, r.emi, 8 * r.ncols, cudaMemcpyDeviceToHost, c->stream));
            if (col_cf_app_h)
                TT_CUDA(cudaMemcpyAsync(col_cf_app_h, r.emf, r.ncols, cudaMemcpyDeviceToHost, c->stream));
        }
        TT_CUDA(cudaStreamSynchronize(c->stream));
        if (nh0) *nh0 = r.nh0;
        if (essential) *essential = r.essential;
        if (ncols) *ncols = r.ncols;
        if (nedges) *nedges = r.m;
    });
}

int tt_dense_redzed_h(tt_ctx* c, const float* x_h, uint32_t n, uint32_t dim, int kind, float p, float* thr_inout,
                      float* mat_h, float* diam_h, int32_t* verts_h, uint64_t cap, uint64_t* count) {
    return tt_dense_redzed_pred_h(c, x_h, n, dim, kind, p, thr_inout, mat_h, diam_h, verts_h, cap, count, nullptr);
}

int tt_dense_redzed_pred_h(tt_ctx* c, const float* x_h, uint32_t n, uint32_t dim, int kind, float p,
                           float* thr_inout, float* mat_h, float* diam_h, int32_t* verts_h, uint64_t cap,
                           uint64_t* count, uint64_t* leftover_h) {
    return guard(c, [&] {
        check_metric(kind, p);
        if (!thr_inout || !count) invalid("gb300: null output");
        const float t = *thr_inout;
        if (std::isnan(t) || t < 0.0f) invalid("persistence: threshold must be non-negative or +inf");
        check_dense_budget(c, n);
        f32* x = c->arena.get<f32>(S_PTS, u64(n) * dim + 1);
        if (n) TT_CUDA(cudaMemcpyAsync(x, x_h, sizeof(f32) * n * dim, cudaMemcpyHostToDevice, c->stream));
        check_finite_dev(c, x, u64(n) * dim);
        f32* mat = c->arena.get<f32>(S_MAT, u64(n) * n + 1);
        u32* rowmax = c->arena.get<u32>(S_ROWMAX, u64(n) + 1);
        dense_matrix(c, x, n, dim, kind, p, mat, std::isinf(t) ? rowmax : nullptr);
        float thr = t;
        if (std::isinf(t) && n) {
            min_bits(c, rowmax, n, rowmax + n);
            u32 b = 0;
            TT_CUDA(cudaMemcpyAsync(&b, rowmax + n, 4, cudaMemcpyDeviceToHost, c->stream));
            TT_CUDA(cudaStreamSynchronize(c->stream));
            thr = bitsf(b);
        }
        *thr_inout = thr;
        f32* d = nullptr;
        int32_t* v = nullptr;
        const u64 m = n ? redzed_edges_owned(c, Complex{mat, nullptr, nullptr, nullptr, n, thr}, &d, &v) : 0;
        *count = m;
        if (mat_h && n)
            TT_CUDA(cudaMemcpyAsync(mat_h, mat, sizeof(f32) * n * n, cudaMemcpyDeviceToHost, c->stream));
        if (m > cap) {
            TT_CUDA(cudaStreamSynchronize(c->stream));
            throw Error(TT_ERR_LENGTH, "gb300: edge list exceeds the output capacity");
        }
        if (m && diam_h) TT_CUDA(cudaMemcpyAsync(diam_h, d, 4 * m, cudaMemcpyDeviceToHost, c->stream));
        if (m && verts_h) TT_CUDA(cudaMemcpyAsync(verts_h, v, 8 * m, cudaMemcpyDeviceToHost, c->stream));
        if (leftover_h && n) {
            const u64 words = u64(n) * ((n + 63) / 64);
            auto* bits = c->arena.get<unsigned long long>(S_MISC1, words);
            redzed_leftover(c, mat, n, thr, bits);
            TT_CUDA(cudaMemcpyAsync(leftover_h, bits, 8 * words, cudaMemcpyDeviceToHost, c->stream));
        }
        TT_CUDA(cudaStreamSynchronize(c->stream));
    });
}

int tt_redzed_leftover_h(tt_ctx* c, const float* mat_dev, uint32_t n, float thr, uint64_t* leftover_h) {
    return guard(c, [&] {
        if (!leftover_h || (n && !mat_dev)) invalid("gb300: null buffer");
        if (std::isnan(thr) || thr < 0.0f) invalid("persistence: threshold must be non-negative or +inf");
        if (!n) return;
        const u64 words = u64(n) * ((n + 63) / 64);
        auto* bits = c->arena.get<unsigned long long>(S_MISC1, words);
        redzed_leftover(c, mat_dev, n, thr, bits);
        TT_CUDA(cudaMemcpyAsync(leftover_h, bits, 8 * words, cudaMemcpyDeviceToHost, c->stream));
        TT_CUDA(cudaStreamSynchronize(c->stream));
    });
}

int tt_graph_redzed_h(tt_ctx* c, const uint64_t* rp_h, const uint32_t* ci_h, const float* w_h, uint32_t n,
                      float thr, float* diam_h, int32_t* verts_h, uint64_t cap, uint64_t* count) {
    return guard(c, [&] {
        if (!count || (n && !rp_h)) invalid("gb300: null buffer");
        if (std::isnan(thr) || thr < 0.0f) invalid("persistence: threshold must be non-negative or +inf");
        const u64 nnz = n ? rp_h[n] : 0;
        u64* rp = c->arena.get<u64>(S_OUT0, u64(n) + 1);
        u32* ci = c->arena.get<u32>(S_OUT1, nnz + 1);
        f32* w = c->arena.get<f32>(S_OUT2, nnz + 1);
        if (n) TT_CUDA(cudaMemcpyAsync(rp, rp_h, 8 * (u64(n) + 1), cudaMemcpyHostToDevice, c->stream));
        if (nnz) {
            TT_CUDA(cudaMemcpyAsync(ci, ci_h, 4 * nnz, cudaMemcpyHostToDevice, c->stream));
            TT_CUDA(cudaMemcpyAsync(w, w_h, 4 * nnz, cudaMemcpyHostToDevice, c->stream));
        }
        f32* d = nullptr;
        int32_t* v = nullptr;
        const u64 m = n ? redzed_edges_owned(c, Complex{nullptr, rp, ci, w, n, thr}, &d, &v) : 0;
        *count = m;
        if (m > cap) {
            TT_CUDA(cudaStreamSynchronize(c->stream));
            throw Error(TT_ERR_LENGTH, "gb300: edge list exceeds the output capacity");
        }
        if (m && diam_h) TT_CUDA(cudaMemcpyAsync(diam_h, d, 4 * m, cudaMemcpyDeviceToHost, c->stream));
        if (m && verts_h) TT_CUDA(cudaMemcpyAsync(verts_h, v, 8 * m, cudaMemcpyDeviceToHost, c->stream));
        TT_CUDA(cudaStreamSynchronize(c->stream));
    });
}

int tt_parse_points_h(tt_ctx* c, const char* text_h, uint64_t bytes, float* pts_h, uint64_t cap, uint32_t* n,
                      uint32_t* dim) {
    return guard(c, [&] {
        if (!n || !dim || (bytes && !text_h) || (cap && !pts_h)) invalid("gb300: null argument");
        parse_points(c, text_h, bytes, pts_h, cap, n, dim);
    });
}

}  // extern "C"
