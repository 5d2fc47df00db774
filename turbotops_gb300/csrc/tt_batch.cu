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
//   k_batch_rowcount + scan   kept pairs per row and their offsets (the
//                   total kept count stays on the device)
//   k_batch_edges   the kept edges of every cloud, compacted, as 64-bit keys
//                     cloud << (31 + ib) | d bits << ib | index
//                   in (cloud, index) order, so one stable radix sort of the
//                   bits above the index field (cloud and d: 40 bits for 512
//                   clouds, four passes) orders all clouds at once by
//                   (cloud, d, index); the sort reads its key count from the
//                   device and skips the tiles beyond it
//   k_batch_emit    EdgeList (diameter, vertex pair) + per-cloud offsets
// Buffers are sized for the worst case (every pair kept), so no step reads a
// count back to the host and the whole sequence is captured into a CUDA
// graph once and replayed.
#include <cmath>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "tt_dense_tile.cuh"

namespace tt {

namespace {

// Square distance tiles of T x T on and above each cloud's diagonal, 256
// threads (tt_dense_tile.cuh: each computed once, an off-diagonal tile
// written twice, row maxima folded); T is picked per batch by the autotuner
// below.
constexpr int BT_THREADS = 32 * dtile::kWarps;
struct TileShape {
    int r, c;
};
constexpr TileShape kShapes[] = {{32, 32}, {64, 64}, {96, 96}};
constexpr int kNumShapes = int(sizeof(kShapes) / sizeof(kShapes[0]));

struct Tile {
    u32 cloud, i0, j0;
};

// Persistent CTAs pull tiles of every cloud from one work list (uneven
// clouds balance themselves). DIM > 0: the dimension at compile time; 0: any.
template <int KIND, int T, int DIM>
__global__ void __launch_bounds__(BT_THREADS)
k_batch_dense(const f32* __restrict__ x, const u64* __restrict__ pt_off, const u64* __restrict__ mat_off,
              const u32* __restrict__ sizes, const Tile* __restrict__ tiles, u32 ntiles, u32 dim, f32 p,
              f32* __restrict__ mats, u32* __restrict__ rowmax, u32* __restrict__ next) {
    __shared__ dtile::Smem<T> sm;
    __shared__ u32 tile_id;
    for (;;) {
        if (threadIdx.x == 0) tile_id = atomicAdd(next, 1u);
        __syncthreads();
        const u32 t = tile_id;   // read before sym_tile's first barrier; rewritten after its last
        if (t >= ntiles) break;
        const Tile tl = tiles[t];
        const u64 po = pt_off[tl.cloud];
        dtile::sym_tile<KIND, DIM, false, T>(x + po * dim, sizes[tl.cloud], dim, p, mats + mat_off[tl.cloud],
                                             rowmax + po, tl.i0, tl.j0, sm);
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

// Kept pairs (j < i, d <= the cloud's radius) per row: one warp per row of
// one cloud (rows listed globally), the count into row_cnt.
__global__ void k_batch_rowcount(const f32* __restrict__ mats, const u64* __restrict__ mat_off,
                                 const u32* __restrict__ sizes, const u64* __restrict__ pt_off,
                                 const u32* __restrict__ row_cloud, u64 rows, const u32* __restrict__ radius,
                                 u64* __restrict__ row_cnt) {
    const int lane = threadIdx.x & 31;
    const u64 warps = (u64(gridDim.x) * blockDim.x) >> 5;
    for (u64 r = (u64(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; r < rows; r += warps) {
        const u32 c = row_cloud[r];
        const u32 n = sizes[c];
        const u32 i = u32(r - pt_off[c]);
        const f32 thr = __uint_as_float(radius[c]);
        const f32* row = mats + mat_off[c] + u64(i) * n;
        u64 kept = 0;
#pragma unroll 4
        for (u32 j0 = 0; j0 < i; j0 += 32) {   // (unrolled: several row loads in flight)
            const u32 j = j0 + lane;
            kept += __popc(__ballot_sync(0xffffffffu, j < i && row[j] <= thr));
        }
        if (lane == 0) row_cnt[r] = kept;
    }
}

// The kept pairs written compacted, at row_off[row] + rank in the row: the
// array runs over (cloud, index) ascending (rows ascending, j ascending in a
// row), so a stable sort on the bits above the index field alone orders it
// by (cloud, d, index). Key: cloud << (31 + ib) | d bits << ib | index.
__global__ void k_batch_edges(const f32* __restrict__ mats, const u64* __restrict__ mat_off,
                              const u32* __restrict__ sizes, const u64* __restrict__ pt_off,
                              const u32* __restrict__ row_cloud, u64 rows, const u32* __restrict__ radius, int ib,
                              const u64* __restrict__ row_off, u64* __restrict__ keys, u64* __restrict__ per_cloud) {
    const int lane = threadIdx.x & 31;
    const u64 warps = (u64(gridDim.x) * blockDim.x) >> 5;
    for (u64 r = (u64(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; r < rows; r += warps) {
        const u32 c = row_cloud[r];
        const u32 n = sizes[c];
        const u32 i = u32(r - pt_off[c]);
        const f32 thr = __uint_as_float(radius[c]);
        const f32* row = mats + mat_off[c] + u64(i) * n;
        const u64 rbase = u64(i) * (i - 1) / 2;
        u64 pos = row_off[r];
#pragma unroll 4
        for (u32 j0 = 0; j0 < i; j0 += 32) {
            const u32 j = j0 + lane;
            const f32 d = j < i ? row[j] : INFINITY;
            const bool keep = j < i && d <= thr;
            const u32 bal = __ballot_sync(0xffffffffu, keep);
            if (keep)
                keys[pos + __popc(bal & ((1u << lane) - 1u))] =
                    (u64(c) << (31 + ib)) | (u64(__float_as_uint(d)) << ib) | (rbase + j);
            pos += __popc(bal);
        }
        const u64 kept = pos - row_off[r];
        if (lane == 0 && kept) atomicAdd((unsigned long long*)&per_cloud[c], (unsigned long long)kept);
    }
}

// Exclusive scan of the per-cloud edge counts (one CTA; clouds <= 65536),
// and the segmented sort's tiles of the kept keys: cloud c's ceil(count /
// kSegTileKeys) tiles after the previous clouds', their digit counts at 256
// per tile in the same order; *ntiles = the list's length.
__global__ void k_batch_offsets(const u64* __restrict__ per_cloud, u32 clouds, u64* __restrict__ off,
                                SegTile* __restrict__ tiles, u32* __restrict__ ntiles) {
    __shared__ u64 part[1024];
    __shared__ u32 tpart[1024];
    const u32 t = threadIdx.x;
    const u32 per = (clouds + blockDim.x - 1) / blockDim.x;
    u64 s = 0;
    u32 ts = 0;
    for (u32 c = t * per; c < min(clouds, (t + 1) * per); ++c) {
        s += per_cloud[c];
        ts += u32((per_cloud[c] + kSegTileKeys - 1) / kSegTileKeys);
    }
    part[t] = s;
    tpart[t] = ts;
    __syncthreads();
    if (t == 0) {
        u64 run = 0;
        u32 trun = 0;
        for (u32 q = 0; q < blockDim.x; ++q) {
            const u64 v = part[q];
            const u32 tv = tpart[q];
            part[q] = run;
            tpart[q] = trun;
            run += v;
            trun += tv;
        }
    }
    __syncthreads();
    u64 run = part[t];
    u32 trun = tpart[t];
    for (u32 c = t * per; c < min(clouds, (t + 1) * per); ++c) {
        off[c] = run;
        run += per_cloud[c];
        const u32 tc = u32((per_cloud[c] + kSegTileKeys - 1) / kSegTileKeys);
        for (u32 q = 0; q < tc; ++q) tiles[trun + q] = SegTile{c, q, 256u * trun, tc};
        trun += tc;
    }
    if (t == blockDim.x - 1) {
        off[clouds] = run;
        *ntiles = trun;
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
    // device buffers (one cudaMalloc each, owned)
    f32* x = nullptr;
    f32* mats = nullptr;
    u32* rowmax = nullptr;
    u32* radius = nullptr;
    u64* pt_off = nullptr;
    u64* mat_off = nullptr;
    u64* pair_off = nullptr;   // first key slot of every cloud's pairs
    u32* sizes = nullptr;
    Tile* tiles[kNumShapes] = {};
    u32 ntiles[kNumShapes] = {};
    int shape = 1;                      // index into kShapes
    bool tuned = false, tuned_from_cache = false;
    float tune_ms[kNumShapes] = {};
    u32* row_cloud = nullptr;
    u32* next = nullptr;
    u64* keys = nullptr;
    u64* kbuf = nullptr;       // the sort's other buffer
    u64* row_cnt = nullptr;    // kept pairs per row, then their exclusive scan
    u64* row_off = nullptr;
    unsigned long long* count = nullptr;
    u64* per_cloud = nullptr;
    u64* edge_off = nullptr;
    SegTile* seg_tiles = nullptr;   // the segmented sort's tiles of the kept keys (built on the device)
    u32* seg_ntiles = nullptr;      // ... their number
    u32 nseg_tiles = 0;             // capacity: every cloud's largest key count in tiles
    u64 seg_hist = 0;               // the digit counts' capacity: 256 per tile
    f32* ed = nullptr;
    int32_t* ev = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    u64 graph_kernels = 0;   // kernels one run launches
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

    template <int T, int D>
    void launch_dense_kd(u32 grid, u32 nt, const Tile* tl, cudaStream_t s) {
        switch (kind) {
            case M_L1: k_batch_dense<M_L1, T, D><<<grid, BT_THREADS, 0, s>>>(x, pt_off, mat_off, sizes, tl, nt, dim, p, mats, rowmax, next); break;
            case M_L2: k_batch_dense<M_L2, T, D><<<grid, BT_THREADS, 0, s>>>(x, pt_off, mat_off, sizes, tl, nt, dim, p, mats, rowmax, next); break;
            case M_LINF: k_batch_dense<M_LINF, T, D><<<grid, BT_THREADS, 0, s>>>(x, pt_off, mat_off, sizes, tl, nt, dim, p, mats, rowmax, next); break;
            default: k_batch_dense<M_LP, T, D><<<grid, BT_THREADS, 0, s>>>(x, pt_off, mat_off, sizes, tl, nt, dim, p, mats, rowmax, next); break;
        }
    }
    template <int T>
    void launch_dense_t(int si, cudaStream_t s) {
        const u32 nt = ntiles[si];
        const u32 grid = u32(std::max<u64>(1, std::min<u64>(nt, u64(owner->sms) * 8)));
        const Tile* tl = tiles[si];
        if (dim == 3) launch_dense_kd<T, 3>(grid, nt, tl, s);
        else launch_dense_kd<T, 0>(grid, nt, tl, s);
        TT_LAUNCH("k_batch_dense");
    }
    void launch_dense(int si, cudaStream_t s) {
        switch (si) {
            case 0: launch_dense_t<32>(si, s); break;
            case 1: launch_dense_t<64>(si, s); break;
            default: launch_dense_t<96>(si, s); break;
        }
    }

    // The autotuner: every tile shape times the distance pass once on this
    // batch (CUDA events on the batch's stream, after one untimed pass that
    // loads the kernels); the fastest serves every later run. The pick is
    // cached per (metric, dimension, cloud count, size classes), so later
    // batches of the same kind skip the timing.
    void tune() {
        static std::mutex mu;
        static std::map<std::string, int> cache;
        std::string key = std::to_string(kind) + "/" + std::to_string(dim) + "/" + std::to_string(clouds) + "/" +
                          std::to_string(maxn >> 6) + "/" + std::to_string(total_pts >> 12);
        {
            std::lock_guard<std::mutex> l(mu);
            auto it = cache.find(key);
            if (it != cache.end()) {
                shape = it->second;
                tuned_from_cache = true;
                return;
            }
        }
        cudaStream_t s = sctx.stream;
        cudaEvent_t e0, e1;
        TT_CUDA(cudaEventCreate(&e0));
        TT_CUDA(cudaEventCreate(&e1));
        float best = 0;
        int pick = 1;
        for (int si = 0; si < kNumShapes; ++si) {
            for (int rep = 0; rep < 2; ++rep) {
                TT_CUDA(cudaMemsetAsync(rowmax, 0, total_pts * sizeof(u32), s));
                TT_CUDA(cudaMemsetAsync(next, 0, sizeof(u32), s));
                TT_CUDA(cudaEventRecord(e0, s));
                launch_dense(si, s);
                TT_CUDA(cudaEventRecord(e1, s));
                sctx.launches += 1;
            }
            TT_CUDA(cudaEventSynchronize(e1));
            float ms = 0;
            TT_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            tune_ms[si] = ms;
            if (si == 0 || ms < best) {
                best = ms;
                pick = si;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        shape = pick;
        std::lock_guard<std::mutex> l(mu);
        cache[key] = pick;
    }

    void enqueue() {
        cudaStream_t s = sctx.stream;
        TT_CUDA(cudaMemsetAsync(rowmax, 0, total_pts * sizeof(u32), s));
        TT_CUDA(cudaMemsetAsync(radius, 0xff, clouds * sizeof(u32), s));
        TT_CUDA(cudaMemsetAsync(next, 0, sizeof(u32), s));
        TT_CUDA(cudaMemsetAsync(count, 0, sizeof(unsigned long long), s));
        TT_CUDA(cudaMemsetAsync(per_cloud, 0, clouds * sizeof(u64), s));
        launch_dense(shape, s);

        const u32 g2 = u32(std::min<u64>((total_pts + 255) / 256, u64(owner->sms) * 16));
        k_batch_radius<<<g2, 256, 0, s>>>(rowmax, row_cloud, total_pts, radius);
        TT_LAUNCH("k_batch_radius");
        const u32 g3 = u32(std::min<u64>((total_pts * 32 + 255) / 256, u64(owner->sms) * 32));
        k_batch_rowcount<<<g3, 256, 0, s>>>(mats, mat_off, sizes, pt_off, row_cloud, total_pts, radius, row_cnt);
        TT_LAUNCH("k_batch_rowcount");
        scan_exclusive<u64>(&sctx, row_cnt, row_off, total_pts, reinterpret_cast<u64*>(count), 0);
        k_batch_edges<<<g3, 256, 0, s>>>(mats, mat_off, sizes, pt_off, row_cloud, total_pts, radius, ib, row_off,
                                         keys, per_cloud);
        TT_LAUNCH("k_batch_edges");
        k_batch_offsets<<<1, 1024, 0, s>>>(per_cloud, clouds, edge_off, seg_tiles, seg_ntiles);
        TT_LAUNCH("k_batch_offsets");
        // every cloud's kept keys on their own (they are contiguous, clouds
        // in order), by the distance bits alone (stable: ties keep the index
        // order): four 8-bit passes, the cloud bits need none
        const bool swapped =
            radix_sort_segments(&sctx, keys, kbuf, edge_off, seg_tiles, seg_ntiles, nseg_tiles, seg_hist, 31, ib);
        const u32 g4 = u32(std::min<u64>((total_pairs + 255) / 256, u64(owner->sms) * 32));
        k_batch_emit<<<g4, 256, 0, s>>>(swapped ? kbuf : keys, count, ib, ed, ev);
        TT_LAUNCH("k_batch_emit");
        sctx.launches += 6;
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
        std::vector<Tile> tiles[kNumShapes];
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
            for (int si = 0; si < kNumShapes; ++si)   // the tiles on and above the diagonal
                for (u32 i0 = 0; i0 < n; i0 += u32(kShapes[si].r))
                    for (u32 j0 = i0; j0 < n; j0 += u32(kShapes[si].c)) tiles[si].push_back(Tile{q, i0, j0});
            for (u32 i = 0; i < n; ++i) row_cloud.push_back(q);
        }
        // the segmented sort's capacity: every cloud's largest key count
        // (every pair kept) in tiles of kSegTileKeys, 256 digit counts a tile
        u64 seg_cap = 0;
        for (u32 q = 0; q < clouds; ++q) seg_cap += div_up(u64(sizes_h[q]) * (sizes_h[q] - 1) / 2, u64(kSegTileKeys));
        if (256 * seg_cap >= (1ull << 32)) invalid("gb300: batch too large for the segmented sort's counts");
        b->ib = std::max(1, Batch::bits_for(u64(b->maxn) * (b->maxn - 1) / 2 + 1));
        if (b->ib + 31 + Batch::bits_for(clouds) > 64)
            invalid("gb300: batch too large for 64-bit edge keys (clouds x largest cloud)");
        b->total_pts = pt_off[clouds];
        b->total_mat = mat_off[clouds];
        b->total_pairs = std::max<u64>(pairs, 1);
        b->x = b->alloc<f32>(b->total_pts * dim);
        b->mats = b->alloc<f32>(b->total_mat);
        b->rowmax = b->alloc<u32>(b->total_pts);
        b->radius = b->alloc<u32>(clouds);
        b->pt_off = b->alloc<u64>(clouds + 1);
        b->mat_off = b->alloc<u64>(clouds + 1);
        b->pair_off = b->alloc<u64>(clouds + 1);
        b->sizes = b->alloc<u32>(clouds);
        for (int si = 0; si < kNumShapes; ++si) {
            b->ntiles[si] = u32(tiles[si].size());
            b->tiles[si] = b->alloc<Tile>(tiles[si].size());
        }
        b->row_cloud = b->alloc<u32>(row_cloud.size());
        b->next = b->alloc<u32>(1);
        b->keys = b->alloc<u64>(b->total_pairs);
        b->kbuf = b->alloc<u64>(b->total_pairs);
        b->row_cnt = b->alloc<u64>(b->total_pts);
        b->row_off = b->alloc<u64>(b->total_pts);
        b->count = b->alloc<unsigned long long>(1);
        b->per_cloud = b->alloc<u64>(clouds);
        b->edge_off = b->alloc<u64>(clouds + 1);
        b->nseg_tiles = u32(seg_cap);
        b->seg_hist = 256 * seg_cap;
        b->seg_tiles = b->alloc<SegTile>(seg_cap);
        b->seg_ntiles = b->alloc<u32>(1);
        b->ed = b->alloc<f32>(b->total_pairs);
        b->ev = b->alloc<int32_t>(2 * b->total_pairs);
        cudaStream_t s = b->sctx.stream;
        TT_CUDA(cudaMemcpyAsync(b->pt_off, pt_off.data(), 8 * (clouds + 1), cudaMemcpyHostToDevice, s));
        TT_CUDA(cudaMemcpyAsync(b->mat_off, mat_off.data(), 8 * (clouds + 1), cudaMemcpyHostToDevice, s));
        TT_CUDA(cudaMemcpyAsync(b->pair_off, pair_off.data(), 8 * (clouds + 1), cudaMemcpyHostToDevice, s));
        TT_CUDA(cudaMemcpyAsync(b->sizes, sizes_h, 4 * clouds, cudaMemcpyHostToDevice, s));
        for (int si = 0; si < kNumShapes; ++si)
            TT_CUDA(cudaMemcpyAsync(b->tiles[si], tiles[si].data(), sizeof(Tile) * tiles[si].size(),
                                    cudaMemcpyHostToDevice, s));
        TT_CUDA(cudaMemcpyAsync(b->row_cloud, row_cloud.data(), 4 * row_cloud.size(), cudaMemcpyHostToDevice, s));
        // size the sort's and the row scan's scratch outside any capture
        radix_reserve_entries(&b->sctx, b->seg_hist);
        // the row scan's levels (64-bit entries: four times as many 32-bit
        // entries reserve at least their bytes at every level)
        radix_reserve_entries(&b->sctx, 4 * b->total_pts);
        TT_CUDA(cudaStreamSynchronize(s));
    } catch (...) {
        b->release();
        delete b;
        throw;
    }
    return b;
}

void batch_run(Batch* b) {
    if (!b->tuned) {   // the first run: pick the tile shape on this batch's points
        b->tune();
        b->tuned = true;
    }
    if (!b->use_graph) {
        const u64 before = b->sctx.launches;
        b->enqueue();
        b->graph_kernels = b->sctx.launches - before;
        return;
    }
    if (!b->exec) {
        TT_CUDA(cudaStreamBeginCapture(b->sctx.stream, cudaStreamCaptureModeThreadLocal));
        try {
            const u64 before = b->sctx.launches;
            b->enqueue();
            b->graph_kernels = b->sctx.launches - before;
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

int tt_batch_tuning(tt_batch* bh, uint32_t* tile_rows, uint32_t* tile_cols, float* shape_ms, uint32_t* shapes,
                    int* from_cache) {
    Batch* b = reinterpret_cast<Batch*>(bh);
    if (!b) return TT_ERR_INVALID;
    if (tile_rows) *tile_rows = u32(kShapes[b->shape].r);
    if (tile_cols) *tile_cols = u32(kShapes[b->shape].c);
    if (shapes) *shapes = u32(kNumShapes);
    if (shape_ms)
        for (int si = 0; si < kNumShapes; ++si) shape_ms[si] = b->tune_ms[si];
    if (from_cache) *from_cache = b->tuned_from_cache ? 1 : 0;
    return TT_OK;
}

int tt_batch_run(tt_batch* bh, int wait) {
    Batch* b = reinterpret_cast<Batch*>(bh);
    if (!b) return TT_ERR_INVALID;
    try {
        TT_CUDA(cudaSetDevice(b->owner->device));
        batch_run(b);
        b->owner->launches += b->graph_kernels;   // the kernels one run launches
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
