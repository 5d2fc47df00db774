// tt_topo.cu — persistence pairs with their critical edges for a batch of
// clouds, and the adjoint that scatters dL/d(birth, death) onto coordinates.
//
// No counterpart in the reference (its Barcode keeps values only,
// rips.hpp:52-67). Forward: for every cloud the GPU runs the dense front end
// (distances, enclosing radius, dim0); host threads run compute_pairs(1) for
// the clouds whose front end is done while the GPU works on the next ones,
// recording each bar's critical
// simplices; each bar value is then the length of one edge:
//   H0 death   the spanning-tree edge that merged two components
//   H1 birth   the column's edge
//   H1 death   the longest edge of the pivot triangle (the edge whose length
//              equals the death value; unique on tie-free input)
// Adjoint: dL/dx_u += g * dd(u,v)/dx_u, dL/dx_v -= the same, for every
// critical edge (u, v) with upstream gradient g, where for
//   L2   dd/dx_u = (x_u - x_v) / d
//   L1   sign(x_u - x_v)
//   Linf e_k* sign(x_u,k* - x_v,k*), k* the first coordinate of largest |diff|
//   Lp   sign(diff_k) (|diff_k| / d)^(p - 1)
// one thread per edge, float atomics into the gradient.
#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <cstdlib>
#include <mutex>
#include <thread>
#include <vector>

#include "tt_internal.cuh"
#include "tt_metric.cuh"
#include "tt_reduce.h"

namespace tt {

namespace {

constexpr u32 NOV = 0xffffffffu;

__global__ void k_topo_adjoint(const f32* __restrict__ x, u32 dim, int kind, f32 p, const u32* __restrict__ edges,
                               const f32* __restrict__ g, u64 m, f32* __restrict__ grad) {
    for (u64 e = u64(blockIdx.x) * blockDim.x + threadIdx.x; e < m; e += u64(gridDim.x) * blockDim.x) {
        const u32 u = edges[2 * e], v = edges[2 * e + 1];
        const f32 ge = g[e];
        if (u == NOV || v == NOV || ge == 0.0f || u == v) continue;
        const f32* xu = x + u64(u) * dim;
        const f32* xv = x + u64(v) * dim;
        f32 s = 0.0f, mx = 0.0f;
        u32 kmax = 0;
        for (u32 k = 0; k < dim; ++k) {
            const f32 d = xu[k] - xv[k];
            const f32 a = fabsf(d);
            if (a > mx) {
                mx = a;
                kmax = k;
            }
            if (kind == M_L2) s = fmaf(d, d, s);
            else if (kind == M_LP) s += powf(a, p);
        }
        f32 dd = kind == M_L2 ? sqrtf(s) : kind == M_LP ? powf(s, 1.0f / p) : 0.0f;
        if ((kind == M_L2 || kind == M_LP) && !(dd > 0.0f)) continue;
        for (u32 k = 0; k < dim; ++k) {
            const f32 d = xu[k] - xv[k];
            f32 w;
            if (kind == M_L2) w = d / dd;
            else if (kind == M_L1) w = d > 0.0f ? 1.0f : (d < 0.0f ? -1.0f : 0.0f);
            else if (kind == M_LINF) w = k == kmax ? (d > 0.0f ? 1.0f : (d < 0.0f ? -1.0f : 0.0f)) : 0.0f;
            else w = (d > 0.0f ? 1.0f : (d < 0.0f ? -1.0f : 0.0f)) * powf(fabsf(d) / dd, p - 1.0f);
            if (w != 0.0f) {
                atomicAdd(&grad[u64(u) * dim + k], ge * w);
                atomicAdd(&grad[u64(v) * dim + k], -ge * w);
            }
        }
    }
}

void decode2(u64 idx, u32& a, u32& b) {   // a > b
    u64 v = u64((1.0 + std::sqrt(1.0 + 8.0 * double(idx))) * 0.5);
    while (v * (v - 1) / 2 > idx) --v;
    while ((v + 1) * v / 2 <= idx) ++v;
    a = u32(v);
    b = u32(idx - v * (v - 1) / 2);
}

void decode3(u64 idx, u32 n, u32& c0, u32& c1, u32& c2) {   // c0 > c1 > c2
    u32 lo = 2, hi = n;
    while (hi - lo > 1) {   // largest v with C(v, 3) <= idx
        const u32 mid = lo + (hi - lo) / 2;
        if (u64(mid) * (mid - 1) * (mid - 2) / 6 <= idx) lo = mid;
        else hi = mid;
    }
    c0 = lo;
    decode2(idx - u64(lo) * (lo - 1) * (lo - 2) / 6, c1, c2);
}

struct Cloud {
    u32 n = 0;
    u64 off = 0;
    f32 thr = 0;
    std::vector<f32> mat, h0d, cd;
    std::vector<u64> h0e, ci, emi;
    std::vector<u8> emf;
    host::Bars bars;
};

// Hands clouds from the thread that runs their device front end to the
// threads that reduce them: a cloud is published once its outputs are on the
// host, and reducers take published clouds in order, so the reductions of the
// first clouds overlap the front end of the later ones and a thread that
// finishes early takes the next cloud. Each cloud's reduction is independent
// of the others, so the bars do not depend on the schedule.
struct CloudQueue {
    std::mutex m;
    std::condition_variable cv;
    u32 count, ready = 0, next = 0;
    bool stop = false;
    explicit CloudQueue(u32 c) : count(c) {}
    // the next cloud to reduce; count when none is left (or after stop)
    u32 take() {
        std::unique_lock<std::mutex> lk(m);
        cv.wait(lk, [&] { return stop || next < ready || next >= count; });
        if (stop || next >= count) return count;
        return next++;
    }
    void publish(u32 q) {
        {
            std::lock_guard<std::mutex> lk(m);
            ready = q + 1;
        }
        cv.notify_all();
    }
    void halt() {
        {
            std::lock_guard<std::mutex> lk(m);
            stop = true;
        }
        cv.notify_all();
    }
};

}  // namespace

struct TopoResult {
    tt_topo_out pub{};
    std::vector<u64> h0_off, h1_off;
    std::vector<f32> h0_death, h1_birth, h1_death;
    std::vector<u32> h0_edge, h1_bedge, h1_dedge;
};

}  // namespace tt

using namespace tt;

extern "C" int tt_topo_forward(tt_ctx* c, const float* x, const uint32_t* sizes, uint32_t count, uint32_t dim,
                               int kind, float p, int threads, tt_topo_out** out) {
    if (!c || !out) return TT_ERR_INVALID;
    *out = nullptr;
    try {
        TT_CUDA(cudaSetDevice(c->device));
        if (kind < TT_METRIC_L1 || kind > TT_METRIC_LP) invalid("metric: unknown kind");
        if (kind == TT_METRIC_LP && !(p >= 1.0f)) invalid("metric: p must be in [1, inf]");
        std::vector<Cloud> cl(count);
        // host reducers (the calling thread joins them after the front end)
        u32 nt = threads > 0 ? u32(threads) : std::max(1u, std::thread::hardware_concurrency());
        // threads beyond one per cloud go into each cloud's own reduction
        const unsigned per_cloud = count ? std::max<u32>(1, nt / std::max<u32>(count, 1)) : 1;
        nt = std::min<u32>(nt, std::max<u32>(count, 1));
        CloudQueue queue(count);
        std::vector<std::string> errs(nt);
        auto work = [&](u32 t) {
            try {
                for (u32 q; (q = queue.take()) < count;) {
                    Cloud& C = cl[q];
                    if (C.n == 0) continue;
                    std::vector<host::Entry> cols(C.ci.size());
                    for (u64 i = 0; i < cols.size(); ++i) cols[i] = host::Entry{C.ci[i], C.cd[i]};
                    host::HostComplex hc{C.mat.data(), nullptr, nullptr, nullptr, C.n, C.thr};
                    std::vector<u64> piv;
                    host::ReduceStats st;
                    C.bars = host::compute_pairs(hc, 1, 1, cols, C.emi.data(), C.emf.data(), piv, st, per_cloud);
                }
            } catch (const std::exception& e) {
                errs[t] = e.what();
                queue.halt();
            }
        };
        std::vector<std::thread> pool;
        auto join = [&] {
            for (auto& th : pool) th.join();
            pool.clear();
        };
        // device front end, cloud by cloud; each cloud goes to the reducers
        // once its outputs are on the host
        auto front_end = [&] {
            u64 off = 0;
            for (u32 q = 0; q < count; ++q) {
                Cloud& C = cl[q];
                C.n = sizes[q];
                C.off = off;
                off += C.n;
                if (C.n == 0) {
                    queue.publish(q);
                    continue;
                }
                const u32 n = C.n;
                f32* mat = c->arena.get<f32>(S_MAT, u64(n) * n + 1);
                u32* rowmax = c->arena.get<u32>(S_ROWMAX, u64(n) + 1);
                dense_matrix(c, x + C.off * dim, n, dim, kind, p, mat, rowmax);
                min_bits(c, rowmax, n, rowmax + n);
                u32 b = 0;
                TT_CUDA(cudaMemcpyAsync(&b, rowmax + n, 4, cudaMemcpyDeviceToHost, c->stream));
                TT_CUDA(cudaStreamSynchronize(c->stream));
                C.thr = bitsf(b);
                Complex cx{mat, nullptr, nullptr, nullptr, n, C.thr};
                Dim0Out r;
                dim0(c, cx, 1, r);
                C.mat.resize(u64(n) * n);
                C.h0d.resize(r.nh0);
                C.h0e.resize(r.nh0);
                C.ci.resize(r.ncols);
                C.cd.resize(r.ncols);
                C.emi.resize(r.ncols);
                C.emf.resize(r.ncols);
                TT_CUDA(cudaMemcpyAsync(C.mat.data(), mat, 4 * u64(n) * n, cudaMemcpyDeviceToHost, c->stream));
                if (r.nh0) {
                    TT_CUDA(cudaMemcpyAsync(C.h0d.data(), r.h0, 4 * r.nh0, cudaMemcpyDeviceToHost, c->stream));
                    TT_CUDA(cudaMemcpyAsync(C.h0e.data(), r.h0_edge, 8 * r.nh0, cudaMemcpyDeviceToHost, c->stream));
                }
                if (r.ncols) {
                    TT_CUDA(cudaMemcpyAsync(C.ci.data(), r.cidx, 8 * r.ncols, cudaMemcpyDeviceToHost, c->stream));
                    TT_CUDA(cudaMemcpyAsync(C.cd.data(), r.cd, 4 * r.ncols, cudaMemcpyDeviceToHost, c->stream));
                    TT_CUDA(cudaMemcpyAsync(C.emi.data(), r.emi, 8 * r.ncols, cudaMemcpyDeviceToHost, c->stream));
                    TT_CUDA(cudaMemcpyAsync(C.emf.data(), r.emf, r.ncols, cudaMemcpyDeviceToHost, c->stream));
                }
                TT_CUDA(cudaStreamSynchronize(c->stream));
                queue.publish(q);
            }
        };
        try {
            for (u32 t = 1; t < nt; ++t) pool.emplace_back(work, t);
            front_end();
        } catch (...) {
            queue.halt();
            join();
            throw;
        }
        work(0);
        join();
        for (auto& e : errs)
            if (!e.empty()) throw Error(TT_ERR_INTERNAL, e);
        // pack, with global point ids
        auto* R = new TopoResult;
        R->h0_off.assign(count + 1, 0);
        R->h1_off.assign(count + 1, 0);
        for (u32 q = 0; q < count; ++q) {
            const Cloud& C = cl[q];
            for (u64 i = 0; i < C.h0d.size(); ++i) {
                u32 a, b;
                decode2(C.h0e[i], a, b);
                R->h0_death.push_back(C.h0d[i]);
                R->h0_edge.push_back(u32(C.off + a));
                R->h0_edge.push_back(u32(C.off + b));
            }
            R->h0_off[q + 1] = R->h0_death.size();
            for (u64 i = 0; i < C.bars.birth.size(); ++i) {
                u32 a, b;
                decode2(C.bars.birth_idx[i], a, b);
                R->h1_birth.push_back(C.bars.birth[i]);
                R->h1_death.push_back(C.bars.death[i]);
                R->h1_bedge.push_back(u32(C.off + a));
                R->h1_bedge.push_back(u32(C.off + b));
                u32 du = NOV, dv = NOV;
                if (C.bars.death_idx[i] != kNone) {
                    u32 c0, c1, c2;
                    decode3(C.bars.death_idx[i], C.n, c0, c1, c2);
                    const f32 dd = C.bars.death[i];
                    const f32* M = C.mat.data();
                    if (M[u64(c1) * C.n + c2] == dd) { du = c1; dv = c2; }
                    else if (M[u64(c0) * C.n + c2] == dd) { du = c0; dv = c2; }
                    else { du = c0; dv = c1; }
                    du = u32(C.off + du);
                    dv = u32(C.off + dv);
                }
                R->h1_dedge.push_back(du);
                R->h1_dedge.push_back(dv);
            }
            R->h1_off[q + 1] = R->h1_birth.size();
        }
        tt_topo_out& P = R->pub;
        P.clouds = count;
        P.h0_offset = R->h0_off.data();
        P.h0_death = R->h0_death.data();
        P.h0_edge = R->h0_edge.data();
        P.h1_offset = R->h1_off.data();
        P.h1_birth = R->h1_birth.data();
        P.h1_death = R->h1_death.data();
        P.h1_birth_edge = R->h1_bedge.data();
        P.h1_death_edge = R->h1_dedge.data();
        P.opaque = R;
        *out = &R->pub;
        return TT_OK;
    } catch (const Error& e) {
        c->last_error = e.what();
        return e.status;
    } catch (const std::exception& e) {
        c->last_error = e.what();
        return TT_ERR_INTERNAL;
    }
}

extern "C" void tt_topo_free(tt_topo_out* out) {
    if (!out) return;
    delete static_cast<TopoResult*>(out->opaque);
}

extern "C" int tt_topo_adjoint(tt_ctx* c, const float* x, uint32_t dim, int kind, float p, const uint32_t* edges,
                               const float* grad_d, uint64_t m, float* grad_x) {
    if (!c) return TT_ERR_INVALID;
    try {
        TT_CUDA(cudaSetDevice(c->device));
        if (kind < TT_METRIC_L1 || kind > TT_METRIC_LP) invalid("metric: unknown kind");
        if (m) {
            const u32 grid = u32(std::min<u64>((m + 255) / 256, u64(c->sms) * 16));
            k_topo_adjoint<<<grid, 256, 0, c->stream>>>(x, dim, kind, p, edges, grad_d, m, grad_x);
            TT_LAUNCH("k_topo_adjoint");
            ++c->launches;
        }
        return TT_OK;
    } catch (const Error& e) {
        c->last_error = e.what();
        return e.status;
    } catch (const std::exception& e) {
        c->last_error = e.what();
        return TT_ERR_INTERNAL;
    }
}
