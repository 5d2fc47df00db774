// tt_batch.cu — the dense front end of many clouds at once, replayed from a
// captured CUDA graph.
//
// Replaces, for every cloud of a batch, the front end the reference runs per
// persistence() call on a full-Rips cloud (turbotops.hpp:230-259 with the
// RedZeD engine that auto picks for H1 on dense input): make_dense
// (rips.hpp:391-416), enclosing_radius (:370-380) and build_edges
// (redzed.hpp:545-613, kept edges in (d asc, combinatorial index asc) order).
//
// The batch is one block-diagonal complex:
//   k_batch_dense   persistent CTAs pull 32 x 64 distance tiles of every cloud
//                   from one work list (uneven clouds balance themselves) and
//                   fold row maxima
//   k_batch_radius  per-cloud minimum of the row maxima
//   k_batch_edges   kept edges of every cloud as 64-bit keys
//                     cloud << (31 + ib) | d bits << ib | index
//                   so one radix sort orders all clouds at once
//   k_batch_emit    EdgeList (diameter, vertex pair) + per-cloud offsets
// Buffers are sized for the worst case (every pair kept; unused keys are
// all-ones and sort last), so no step reads a count back to the host and
// the whole sequence is captured into a CUDA graph once and replayed.
#include <cmath>
#include <vector>

#include "tt_internal.cuh"
#include "tt_metric.cuh"

namespace tt {

namespace {

constexpr int BT_R = 32, BT_C = 64, BT_Y = 4;

struct Tile {
    u32 cloud, i0, j0;
};

template <int KIND>
__global__ void __launch_bounds__(BT_C* BT_Y)
k_batch_dense(const f32* __restrict__ x, const u64* __restrict__ pt_off, const u64* __restrict__ mat_off,
              const u32* __restrict__ sizes, const Tile* __restrict__ tiles, u32 ntiles, u32 dim, f32 p,
              f32* __restrict__ mats, u32* __restrict__ rowmax, u32* __restrict__ next) {
    __shared__ u32 smax[BT_R];
    __shared__ u32 tile_id;
    const u32 tx = threadIdx.x, ty = threadIdx.y, tid = ty * BT_C + tx;
    for (;;) {
        if (tid == 0) tile_id = atomicAdd(next, 1u);
        if (tid < BT_R) smax[tid] = 0u;
        __syncthreads();
        const u32 t = tile_id;
        if (t >= ntiles) break;
        const Tile tl = tiles[t];
        const u32 n = sizes[tl.cloud];
        const f32* xc = x + pt_off[tl.cloud] * dim;
        f32* mc = mats + mat_off[tl.cloud];
        const u32 j = tl.j0 + tx;
        for (u32 r = ty; r < BT_R; r += BT_Y) {
            const u32 i = tl.i0 + r;
            if (i >= n) break;
            f32 d = 0.0f;
            if (j < n) {
                d = (i == j) ? 0.0f : metric_dist(KIND, p, Row{xc + u64(i) * dim}, Row{xc + u64(j) * dim}, dim);
                mc[u64(i) * n + j] = d;
            }
            u32 v = __float_as_uint(d);
#pragma unroll
            for (int o = 16; o; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
            if ((tx & 31) == 0) atomicMax(&smax[r], v);
        }
        __syncthreads();
        if (tid < BT_R && tl.i0 + tid < n) atomicMax(&rowmax[pt_off[tl.cloud] + tl.i0 + tid], smax[tid]);
        __syncthreads();
    }
}

// (A cloud's rows are contiguous: a warp whose 32 rows share one cloud takes
// their minimum first and issues one atomic.)
__global__ void k_batch_radius(const u32* __restrict__ rowmax, const u32* __restrict__ row_cloud, u64 rows,
                               u32* __restrict__ radius) {
    const u32 lane = threadIdx.x & 31;
    const u64 stride = u64(gridDim.x) * blockDim.x;
    for (u64 base = u64(blockIdx.x) * blockDim.x + (threadIdx.x & ~31u); base < rows; base += stride) {
        const u64 r = base + lane;   // whole warps iterate together
        const bool ok = r < rows;
        const u32 c = ok ? row_cloud[r] : 0xffffffffu;
        u32 v = ok ? rowmax[r] : 0xffffffffu;
        const u32 c0 = __shfl_sync(0xffffffffu, c, 0);
        if (__all_sync(0xffffffffu, !ok || c == c0)) {
            v = __reduce_min_sync(0xffffffffu, v);
            if (lane == 0) atomicMin(&radius[c0], v);
        } else if (ok) {
            atomicMin(&radius[c], v);
        }
    }
}

// One warp per row of one cloud (rows listed globally).
// Every pair (c, i, j), j < i, owns key slot pair_off[c] + i (i - 1) / 2 + j:
// a kept pair writes its key there (coalesced, no shared counter), the rest
// keep the all-ones fill and sort last.
__global__ void k_batch_edges(const f32* __restrict__ mats, const u64* __restrict__ mat_off,
                              const u64* __restrict__ pair_off, const u32* __restrict__ sizes,
                              const u64* __restrict__ pt_off, const u32* __restrict__ row_cloud, u64 rows,
                              const u32* __restrict__ radius, int ib, u64* __restrict__ keys,
                              u64* __restrict__ per_cloud) {
    const int lane = threadIdx.x & 31;
    const u64 warps = (u64(gridDim.x) * blockDim.x) >> 5;
    for (u64 r = (u64(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; r < rows; r += warps) {
        const u32 c = row_cloud[r];
        const u32 n = sizes[c];
        const u32 i = u32(r - pt_off[c]);
        const f32 thr = __uint_as_float(radius[c]);
        const f32* row = mats + mat_off[c] + u64(i) * n;
        const u64 rbase = u64(i) * (i - 1) / 2;
        u64* slots = keys + pair_off[c] + rbase;
        u64 kept = 0;
        for (u32 j0 = 0; j0 < i; j0 += 32) {
            const u32 j = j0 + lane;
            const f32 d = j < i ? row[j] : INFINITY;
            const bool keep = j < i && d <= thr;
            kept += __popc(__ballot_sync(0xffffffffu, keep));
            if (keep) slots[j] = (u64(c) << (31 + ib)) | (u64(__float_as_uint(d)) << ib) | (rbase + j);
        }
        if (lane == 0 && kept) atomicAdd((unsigned long long*)&per_cloud[c], (unsigned long long)kept);
    }
}

// Exclusive scan of the per-cloud edge counts (one CTA; clouds <= 65536);
// *count = all kept edges.
__global__ void k_batch_offsets(const u64* __restrict__ per_cloud, u32 clouds, u64* __restrict__ off,
                                unsigned long long* __restrict__ count) {
    __shared__ u64 part[1024];
    const u32 t = threadIdx.x;
    const u32 per = (clouds + blockDim.x - 1) / blockDim.x;
    u64 s = 0;
    for (u32 c = t * per; c < min(clouds, (t + 1) * per); ++c) s += per_cloud[c];
    part[t] = s;
    __syncthreads();
    if (t == 0) {
        u64 run = 0;
        for (u32 q = 0; q < blockDim.x; ++q) {
            const u64 v = part[q];
            part[q] = run;
            run += v;
        }
    }
    __syncthreads();
    u64 run = part[t];
    for (u32 c = t * per; c < min(clouds, (t + 1) * per); ++c) {
        off[c] = run;
        run += per_cloud[c];
    }
    if (t == blockDim.x - 1) {
        off[clouds] = run;
        *count = run;
    }
}

__global__ void k_batch_emit(const u64* __restrict__ keys, const unsigned long long* __restrict__ count, int ib,
                             f32* __restrict__ d, int32_t* __restrict__ verts) {
    const u64 m = *count;
    const u64 imask = (1ull << ib) - 1;
    for (u64 e = u64(blockIdx.x) * blockDim.x + threadIdx.x; e < m; e += u64(gridDim.x) * blockDim.x) {
        const u64 k = keys[e];
        u32 a, b;
        decode_edge(k & imask, a, b);
        d[e] = __uint_as_float(u32((k >> ib) & 0x7fffffffu));
        verts[2 * e] = int32_t(b);
        verts[2 * e + 1] = int32_t(a);
    }
}

}  // namespace

struct Batch {
    tt_ctx* owner = nullptr;
    tt_ctx sctx;   // capture stream + own arena for the sort's scratch
    u32 clouds = 0, dim = 0, maxn = 0;
    int kind = 0;
    f32 p = 2.0f;
    int ib = 0;
    u64 total_pts = 0, total_mat = 0, total_pairs = 0;
    u32 ntiles = 0;
    // device buffers (one cudaMalloc each, owned)
    f32* x = nullptr;
    f32* mats = nullptr;
    u32* rowmax = nullptr;
    u32* radius = nullptr;
    u64* pt_off = nullptr;
    u64* mat_off = nullptr;
    u64* pair_off = nullptr;   // first key slot of every cloud's pairs
    u32* sizes = nullptr;
    Tile* tiles = nullptr;
    u32* row_cloud = nullptr;
    u32* next = nullptr;
    u64* keys = nullptr;
    unsigned long long* count = nullptr;
    u64* per_cloud = nullptr;
    u64* edge_off = nullptr;
    f32* ed = nullptr;
    int32_t* ev = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool use_graph = true;
    std::vector<void*> owned;

    template <typename T>
    T* alloc(u64 count) {
        void* p = nullptr;
        const cudaError_t e = cudaMalloc(&p, std::max<u64>(count, 1) * sizeof(T));
        if (e != cudaSuccess) {
            cudaGetLastError();
            throw Error(TT_ERR_LENGTH, "gb300: batch buffers exceed device memory");
        }
        owned.push_back(p);
        return static_cast<T*>(p);
    }

    void enqueue() {
        cudaStream_t s = sctx.stream;
        TT_CUDA(cudaMemsetAsync(rowmax, 0, total_pts * sizeof(u32), s));
        TT_CUDA(cudaMemsetAsync(radius, 0xff, clouds * sizeof(u32), s));
        TT_CUDA(cudaMemsetAsync(next, 0, sizeof(u32), s));
        TT_CUDA(cudaMemsetAsync(count, 0, sizeof(unsigned long long), s));
        TT_CUDA(cudaMemsetAsync(per_cloud, 0, clouds * sizeof(u64), s));
        TT_CUDA(cudaMemsetAsync(keys, 0xff, total_pairs * sizeof(u64), s));
        const dim3 blk(BT_C, BT_Y);
        const u32 grid = u32(std::min<u64>(ntiles, u64(owner->sms) * 8));
        switch (kind) {
            case M_L1: k_batch_dense<M_L1><<<grid, blk, 0, s>>>(x, pt_off, mat_off, sizes, tiles, ntiles, dim, p, mats, rowmax, next); break;
            case M_L2: k_batch_dense<M_L2><<<grid, blk, 0, s>>>(x, pt_off, mat_off, sizes, tiles, ntiles, dim, p, mats, rowmax, next); break;
            case M_LINF: k_batch_dense<M_LINF><<<grid, blk, 0, s>>>(x, pt_off, mat_off, sizes, tiles, ntiles, dim, p, mats, rowmax, next); break;
            default: k_batch_dense<M_LP><<<grid, blk, 0, s>>>(x, pt_off, mat_off, sizes, tiles, ntiles, dim, p, mats, rowmax, next); break;
        }
        TT_LAUNCH("k_batch_dense");
        const u32 g2 = u32(std::min<u64>((total_pts + 255) / 256, u64(owner->sms) * 16));
        k_batch_radius<<<g2, 256, 0, s>>>(rowmax, row_cloud, total_pts, radius);
        TT_LAUNCH("k_batch_radius");
        const u32 g3 = u32(std::min<u64>((total_pts * 32 + 255) / 256, u64(owner->sms) * 32));
        k_batch_edges<<<g3, 256, 0, s>>>(mats, mat_off, pair_off, sizes, pt_off, row_cloud, total_pts, radius, ib,
                                         keys, per_cloud);
        TT_LAUNCH("k_batch_edges");
        k_batch_offsets<<<1, 1024, 0, s>>>(per_cloud, clouds, edge_off, count);
        TT_LAUNCH("k_batch_offsets");
        radix_sort_inplace<u32>(&sctx, keys, nullptr, total_pairs, 31 + ib + bits_for(clouds));
        const u32 g4 = u32(std::min<u64>((total_pairs + 255) / 256, u64(owner->sms) * 32));
        k_batch_emit<<<g4, 256, 0, s>>>(keys, count, ib, ed, ev);
        TT_LAUNCH("k_batch_emit");
        sctx.launches += 5;
    }

    static int bits_for(u64 v) {
        int b = 0;
        while ((1ull << b) < v) ++b;
        return b;
    }

    void release() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
        for (void* q : owned) cudaFree(q);
        owned.clear();
        sctx.arena.release();
        if (sctx.stream) cudaStreamDestroy(sctx.stream);
        sctx.stream = nullptr;
    }
};

Batch* batch_create(tt_ctx* c, const u32* sizes_h, u32 clouds, u32 dim, int kind, f32 p, int use_graph) {
    if (clouds == 0) invalid("gb300: empty batch");
    if (dim == 0) invalid("gb300: dim must be >= 1");
    auto* b = new Batch;
    try {
        b->owner = c;
        b->clouds = clouds;
        b->dim = dim;
        b->kind = kind;
        b->p = p;
        b->use_graph = use_graph != 0;
        b->sctx.device = c->device;
        b->sctx.sms = c->sms;
        TT_CUDA(cudaStreamCreateWithFlags(&b->sctx.stream, cudaStreamNonBlocking));
        std::vector<u64> pt_off(clouds + 1, 0), mat_off(clouds + 1, 0), pair_off(clouds + 1, 0);
        std::vector<Tile> tiles;
        std::vector<u32> row_cloud;
        u64 pairs = 0;
        for (u32 q = 0; q < clouds; ++q) {
            const u32 n = sizes_h[q];
            if (n < 1) invalid("gb300: every cloud needs at least one point");
            b->maxn = std::max(b->maxn, n);
            pt_off[q + 1] = pt_off[q] + n;
            mat_off[q + 1] = mat_off[q] + u64(n) * n;
            pairs += u64(n) * (n - 1) / 2;
            pair_off[q + 1] = pairs;
            for (u32 i0 = 0; i0 < n; i0 += BT_R)
                for (u32 j0 = 0; j0 < n; j0 += BT_C) tiles.push_back(Tile{q, i0, j0});
            for (u32 i = 0; i < n; ++i) row_cloud.push_back(q);
        }
        b->ib = std::max(1, Batch::bits_for(u64(b->maxn) * (b->maxn - 1) / 2 + 1));
        if (b->ib + 31 + Batch::bits_for(clouds) > 64)
            invalid("gb300: batch too large for 64-bit edge keys (clouds x largest cloud)");
        b->total_pts = pt_off[clouds];
        b->total_mat = mat_off[clouds];
        b->total_pairs = std::max<u64>(pairs, 1);
        b->ntiles = u32(tiles.size());
        b->x = b->alloc<f32>(b->total_pts * dim);
        b->mats = b->alloc<f32>(b->total_mat);
        b->rowmax = b->alloc<u32>(b->total_pts);
        b->radius = b->alloc<u32>(clouds);
        b->pt_off = b->alloc<u64>(clouds + 1);
        b->mat_off = b->alloc<u64>(clouds + 1);
        b->pair_off = b->alloc<u64>(clouds + 1);
        b->sizes = b->alloc<u32>(clouds);
        b->tiles = b->alloc<Tile>(tiles.size());
        b->row_cloud = b->alloc<u32>(row_cloud.size());
        b->next = b->alloc<u32>(1);
        b->keys = b->alloc<u64>(b->total_pairs);
        b->count = b->alloc<unsigned long long>(1);
        b->per_cloud = b->alloc<u64>(clouds);
        b->edge_off = b->alloc<u64>(clouds + 1);
        b->ed = b->alloc<f32>(b->total_pairs);
        b->ev = b->alloc<int32_t>(2 * b->total_pairs);
        cudaStream_t s = b->sctx.stream;
        TT_CUDA(cudaMemcpyAsync(b->pt_off, pt_off.data(), 8 * (clouds + 1), cudaMemcpyHostToDevice, s));
        TT_CUDA(cudaMemcpyAsync(b->mat_off, mat_off.data(), 8 * (clouds + 1), cudaMemcpyHostToDevice, s));
        TT_CUDA(cudaMemcpyAsync(b->pair_off, pair_off.data(), 8 * (clouds + 1), cudaMemcpyHostToDevice, s));
        TT_CUDA(cudaMemcpyAsync(b->sizes, sizes_h, 4 * clouds, cudaMemcpyHostToDevice, s));
        TT_CUDA(cudaMemcpyAsync(b->tiles, tiles.data(), sizeof(Tile) * tiles.size(), cudaMemcpyHostToDevice, s));
        TT_CUDA(cudaMemcpyAsync(b->row_cloud, row_cloud.data(), 4 * row_cloud.size(), cudaMemcpyHostToDevice, s));
        // size the sort's scratch outside any capture: the same calls, no graph
        b->sctx.arena.get<u64>(S_SORT_A, b->total_pairs);
        radix_reserve(&b->sctx, b->total_pairs);
        TT_CUDA(cudaStreamSynchronize(s));
    } catch (...) {
        b->release();
        delete b;
        throw;
    }
    return b;
}

void batch_run(Batch* b) {
    if (!b->use_graph) {
        b->enqueue();
        return;
    }
    if (!b->exec) {
        TT_CUDA(cudaStreamBeginCapture(b->sctx.stream, cudaStreamCaptureModeThreadLocal));
        try {
            b->enqueue();
        } catch (...) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(b->sctx.stream, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        TT_CUDA(cudaStreamEndCapture(b->sctx.stream, &b->graph));
        TT_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
    }
    TT_CUDA(cudaGraphLaunch(b->exec, b->sctx.stream));
}

}  // namespace tt

using namespace tt;

extern "C" {

int tt_batch_create(tt_ctx* c, const uint32_t* sizes, uint32_t count, uint32_t dim, int kind, float p,
                    int use_graph, tt_batch** out) {
    if (!c || !out) return TT_ERR_INVALID;
    try {
        TT_CUDA(cudaSetDevice(c->device));
        if (kind < TT_METRIC_L1 || kind > TT_METRIC_LP) invalid("metric: unknown kind");
        if (kind == TT_METRIC_LP && !(p >= 1.0f)) invalid("metric: p must be in [1, inf]");
        *out = reinterpret_cast<tt_batch*>(batch_create(c, sizes, count, dim, kind, p, use_graph));
        return TT_OK;
    } catch (const Error& e) {
        c->last_error = e.what();
        return e.status;
    } catch (const std::exception& e) {
        c->last_error = e.what();
        return TT_ERR_INTERNAL;
    }
}

float* tt_batch_points(tt_batch* b) { return b ? reinterpret_cast<Batch*>(b)->x : nullptr; }

int tt_batch_run(tt_batch* bh, int wait) {
    Batch* b = reinterpret_cast<Batch*>(bh);
    if (!b) return TT_ERR_INVALID;
    try {
        TT_CUDA(cudaSetDevice(b->owner->device));
        batch_run(b);
        b->owner->launches += 5 + 8 * 5;   // the graph's kernels (dense, radius, edges, offsets, emit, 8 sort passes)
        if (wait) TT_CUDA(cudaStreamSynchronize(b->sctx.stream));
        return TT_OK;
    } catch (const Error& e) {
        b->owner->last_error = e.what();
        return e.status;
    } catch (const std::exception& e) {
        b->owner->last_error = e.what();
        return TT_ERR_INTERNAL;
    }
}

int tt_batch_result(tt_batch* bh, tt_batch_out* out) {
    Batch* b = reinterpret_cast<Batch*>(bh);
    if (!b || !out) return TT_ERR_INVALID;
    out->clouds = b->clouds;
    out->total_points = b->total_pts;
    out->radius_dev = reinterpret_cast<const float*>(b->radius);
    out->edge_offset_dev = b->edge_off;
    out->diam_dev = b->ed;
    out->verts_dev = b->ev;
    out->mats_dev = b->mats;
    out->stream = b->sctx.stream;
    return TT_OK;
}

void tt_batch_destroy(tt_batch* bh) {
    Batch* b = reinterpret_cast<Batch*>(bh);
    if (!b) return;
    cudaSetDevice(b->owner->device);
    if (b->sctx.stream) cudaStreamSynchronize(b->sctx.stream);
    b->release();
    delete b;
}

}  // extern "C"
