// tt_knn.cu — exact all-pairs scans over a point cloud: k nearest neighbours,
// the symmetric kNN graph, the radius graph and the per-round nearest
// foreign neighbour of the complete-graph Borůvka MST.
//
// Replaces graph.hpp knn_lists_exact (:211-225, k-d tree + heap, ties by id),
// knn_graph (:286-304) + CsrGraph::from_rows (core.hpp:113-134),
// radius_graph (:170-201) and the distance scans of mst::h0 (mst.hpp:25-99).
// The reference's k-d tree is an exact accelerator (its pruning is
// conservative, graph.hpp:114-119), so an exhaustive scan with the same
// distance bits and the same (distance, id) order returns the same lists.
//
// One tiled all-pairs scanner (tt_scan.cuh) serves all four.
#include "tt_scan.cuh"

namespace tt {

using scan::KnnOp;
using scan::RadiusCountOp;
using scan::RadiusFillOp;
using scan::ForeignOp;
using scan::scan_all;

namespace {

u32* error_word(tt_ctx* c) {
    u32* e = c->arena.get<u32>(S_MISC2, 4);
    TT_CUDA(cudaMemsetAsync(e, 0, sizeof(u32), c->stream));
    return e;
}

void check_error_word(tt_ctx* c, const u32* e) {
    u32 h = 0;
    TT_CUDA(cudaMemcpyAsync(&h, e, 4, cudaMemcpyDeviceToHost, c->stream));
    TT_CUDA(cudaStreamSynchronize(c->stream));
    if (h & TT_DEV_ERR_TIMEOUT) throw Error(TT_ERR_TIMEOUT, "gb300: a bounded device wait timed out");
}

// --------------------------------------------------------------------------
// Graph assembly kernels.
// --------------------------------------------------------------------------
__global__ void k_knn_pairs(const u32* __restrict__ ids, const f32* __restrict__ d, u32 n, u32 k,
                            u64* __restrict__ keys, u32* __restrict__ vals) {
    const u64 total = u64(n) * k;
    for (u64 e = u64(blockIdx.x) * blockDim.x + threadIdx.x; e < total; e += u64(gridDim.x) * blockDim.x) {
        const u32 i = u32(e / k), j = ids[e];
        const u32 b = __float_as_uint(d[e]);
        keys[2 * e] = (u64(i) << 32) | j;
        vals[2 * e] = b;
        keys[2 * e + 1] = (u64(j) << 32) | i;
        vals[2 * e + 1] = b;
    }
}

__global__ void k_unique_flags(const u64* __restrict__ keys, u64 m, u64* __restrict__ f) {
    for (u64 e = u64(blockIdx.x) * blockDim.x + threadIdx.x; e < m; e += u64(gridDim.x) * blockDim.x)
        f[e] = e == 0 || keys[e] != keys[e - 1];
}

__global__ void k_unique_emit(const u64* __restrict__ keys, const u32* __restrict__ vals, u64 m,
                              const u64* __restrict__ f, const u64* __restrict__ pos, u32* __restrict__ ci,
                              f32* __restrict__ w, u32* __restrict__ rows) {
    for (u64 e = u64(blockIdx.x) * blockDim.x + threadIdx.x; e < m; e += u64(gridDim.x) * blockDim.x) {
        if (!f[e]) continue;
        const u64 o = pos[e];
        ci[o] = u32(keys[e]);
        w[o] = __uint_as_float(vals[e]);
        rows[o] = u32(keys[e] >> 32);
    }
}

// row_ptr from the row of each entry of a row-sorted list
__global__ void k_row_ptr(const u32* __restrict__ rows, u64 nnz, u32 n, u64* __restrict__ rp) {
    for (u64 e = u64(blockIdx.x) * blockDim.x + threadIdx.x; e <= nnz; e += u64(gridDim.x) * blockDim.x) {
        const int64_t lo = e == 0 ? -1 : int64_t(rows[e - 1]);
        const int64_t hi = e == nnz ? int64_t(n) : int64_t(rows[e]);
        for (int64_t r = lo + 1; r <= hi; ++r) rp[r] = e;
    }
}

// ---- symmetric kNN graph without a global sort ------------------------------
// Every list entry (i, j, d) lands in row i and in row j (count, scan,
// atomic fill); each row is then ordered by column with a warp-local rank
// sort and its duplicates (mutual neighbours: same column, same distance
// bits) dropped. Rows longer than kRowSortMax fall back to the global sort.
constexpr u32 kRowSortMax = 2048;
constexpr u32 kWarpRowMax = 128;   // longer rows: one block each (k_graph_rowsort_long)

// Rank of each of a row's L <= 32 * SLOTS entries (slot j of lane l holds
// position 32 j + l) by (column, position), and whether an equal column
// comes earlier, in one pass of shuffles; scattered into the sorted copy.
// Returns the row's distinct columns.
template <int SLOTS>
__device__ __forceinline__ u32 warp_rank_row(const u32* __restrict__ col, const f32* __restrict__ w, u64 b, u32 L,
                                             u32* __restrict__ scol, f32* __restrict__ sw, u32 lane) {
    u32 x[SLOTS], r[SLOTS], e[SLOTS];
    f32 wv[SLOTS];
#pragma unroll
    for (int j = 0; j < SLOTS; ++j) {
        const u32 p = 32u * j + lane;
        x[j] = p < L ? col[b + p] : 0xffffffffu;
        wv[j] = p < L ? w[b + p] : 0.0f;
        r[j] = 0;
        e[j] = 0;
    }
#pragma unroll
    for (int c = 0; c < SLOTS; ++c) {
        if (32u * c >= L) break;   // warp-uniform
        const u32 lim = L - 32u * c < 32u ? L - 32u * c : 32u;
        for (u32 s = 0; s < lim; ++s) {
            const u32 cs = __shfl_sync(0xffffffffu, x[c], s);
#pragma unroll
            for (int j = 0; j < SLOTS; ++j) {
                // position 32 c + s precedes position 32 j + lane?
                const bool before = c < j || (c == j && s < lane);
                r[j] += cs < x[j] || (cs == x[j] && before);
                e[j] += cs == x[j] && before;
            }
        }
    }
    u32 uc = 0;
#pragma unroll
    for (int j = 0; j < SLOTS; ++j) {
        const u32 p = 32u * j + lane;
        if (p < L) {
            scol[b + r[j]] = x[j];
            sw[b + r[j]] = wv[j];
        }
        uc += __popc(__ballot_sync(0xffffffffu, p < L && e[j] == 0));
    }
    return uc;
}

// Row i holds its own list (k entries, slots off[i] .. off[i] + k - 1 in
// list order) and the entries naming i (after them, atomic cursor).
__global__ void k_graph_deg(const u32* __restrict__ ids, u32 n, u32 k, unsigned long long* __restrict__ deg) {
    pdl_wait();
    pdl_trigger();
    const u64 total = u64(n) * k;
    for (u64 e = u64(blockIdx.x) * blockDim.x + threadIdx.x; e < total; e += u64(gridDim.x) * blockDim.x) {
        if (e % k == 0) atomicAdd(&deg[e / k], (unsigned long long)k);
        atomicAdd(&deg[ids[e]], 1ull);
    }
}

__global__ void k_graph_fill(const u32* __restrict__ ids, const f32* __restrict__ d, u32 n, u32 k,
                             const u64* __restrict__ off, u32* __restrict__ cur, u32* __restrict__ col,
                             f32* __restrict__ w) {
    pdl_wait();
    pdl_trigger();
    const u64 total = u64(n) * k;
    for (u64 e = u64(blockIdx.x) * blockDim.x + threadIdx.x; e < total; e += u64(gridDim.x) * blockDim.x) {
        const u32 i = u32(e / k), j = ids[e];
        const f32 de = d[e];
        const u64 a = off[i] + e % k;
        col[a] = j;
        w[a] = de;
        const u64 b = off[j] + k + atomicAdd(&cur[j], 1u);
        col[b] = i;
        w[b] = de;
    }
}

// One warp per row: rank of each entry by (column, position), scattered into
// the sorted copy; ucnt[v] = distinct columns. Rows above kRowSortMax set
// *overflow and are left to the global sort; rows above kWarpRowMax are
// listed (longs[0] = count, then the rows) for k_graph_rowsort_long.
__global__ void k_graph_rowsort(const u64* __restrict__ off, u32 n, const u32* __restrict__ col,
                                const f32* __restrict__ w, u32* __restrict__ scol, f32* __restrict__ sw,
                                unsigned long long* __restrict__ ucnt, u32* __restrict__ overflow,
                                u32* __restrict__ longs) {
    pdl_wait();
    pdl_trigger();
    const int lane = threadIdx.x & 31;
    const u32 warps = (gridDim.x * blockDim.x) >> 5;
    for (u32 v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += warps) {
        const u64 b = off[v];
        const u32 L = u32(off[v + 1] - b);
        if (L > kRowSortMax) {
            if (lane == 0) atomicOr(overflow, 1u);
            continue;
        }
        if (L > kWarpRowMax) {   // k_graph_rowsort_long
            if (lane == 0) longs[1 + atomicAdd(longs, 1u)] = v;
            continue;
        }
        const u32 uc = L <= 32 ? warp_rank_row<1>(col, w, b, L, scol, sw, lane)
                       : L <= 64 ? warp_rank_row<2>(col, w, b, L, scol, sw, lane)
                                 : warp_rank_row<4>(col, w, b, L, scol, sw, lane);
        if (lane == 0) ucnt[v] = uc;
        __syncwarp();
    }
}

// Rows of kWarpRowMax < L <= kRowSortMax entries (hubs: points in many
// lists): one block per row, a bitonic sort of (column << 32 | distance
// bits) in shared memory; duplicates are then identical and adjacent.
constexpr u32 kLongThreads = 256;
__global__ void __launch_bounds__(kLongThreads) k_graph_rowsort_long(const u64* __restrict__ off,
                                                                     const u32* __restrict__ longs,
                                                                     const u32* __restrict__ col,
                                                                     const f32* __restrict__ w, u32* __restrict__ scol,
                                                                     f32* __restrict__ sw,
                                                                     unsigned long long* __restrict__ ucnt) {
    pdl_wait();
    pdl_trigger();
    __shared__ unsigned long long key[kRowSortMax];
    __shared__ u32 uc;
    const u32 tid = threadIdx.x;
    const u32 nl = longs[0];
    for (u32 li = blockIdx.x; li < nl; li += gridDim.x) {
        const u32 v = longs[1 + li];
        const u64 b = off[v];
        const u32 L = u32(off[v + 1] - b);
        u32 P = 1;
        while (P < L) P <<= 1;
        for (u32 i = tid; i < P; i += kLongThreads)
            key[i] = i < L ? (u64(col[b + i]) << 32) | __float_as_uint(w[b + i]) : ~0ull;
        if (tid == 0) uc = 0;
        __syncthreads();
        for (u32 kk = 2; kk <= P; kk <<= 1) {
            for (u32 j = kk >> 1; j > 0; j >>= 1) {
                for (u32 i = tid; i < P; i += kLongThreads) {
                    const u32 ij = i ^ j;
                    if (ij > i) {
                        const unsigned long long x0 = key[i], x1 = key[ij];
                        if ((x0 > x1) == ((i & kk) == 0)) {
                            key[i] = x1;
                            key[ij] = x0;
                        }
                    }
                }
                __syncthreads();
            }
        }
        u32 c = 0;
        for (u32 i = tid; i < L; i += kLongThreads) {
            const unsigned long long x = key[i];
            scol[b + i] = u32(x >> 32);
            sw[b + i] = __uint_as_float(u32(x));
            c += i == 0 || (key[i - 1] >> 32) != (x >> 32);
        }
        atomicAdd(&uc, c);
        __syncthreads();
        if (tid == 0) ucnt[v] = uc;
        __syncthreads();
    }
}

// One warp per row: the distinct columns of the sorted row into the CSR.
// Enqueued before the host has read the overflow flag: with a row left to
// the global sort, the row pointers are meaningless and nothing is written.
__global__ void k_graph_emit(const u64* __restrict__ off, u32 n, const u32* __restrict__ scol,
                             const f32* __restrict__ sw, const u64* __restrict__ rp, u32* __restrict__ ci,
                             f32* __restrict__ wout, const u32* __restrict__ overflow) {
    pdl_wait();
    pdl_trigger();
    if (*overflow) return;
    const int lane = threadIdx.x & 31;
    const u32 warps = (gridDim.x * blockDim.x) >> 5;
    for (u32 v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += warps) {
        const u64 b = off[v];
        const u32 L = u32(off[v + 1] - b);
        u64 o = rp[v];
        for (u32 r0 = 0; r0 < L; r0 += 32) {
            const u32 r = r0 + lane;
            const bool u = r < L && (r == 0 || scol[b + r - 1] != scol[b + r]);
            const u32 bal = __ballot_sync(0xffffffffu, u);
            if (u) {
                const u64 q = o + __popc(bal & ((1u << lane) - 1));
                ci[q] = scol[b + r];
                wout[q] = sw[b + r];
            }
            o += __popc(bal);
        }
    }
}

inline u32 grid_for(u64 work, u32 per_block) {
    const u64 g = (work + per_block - 1) / per_block;
    return u32(std::max<u64>(1, std::min<u64>(g, 64ull * kSMs)));
}

}  // namespace

bool knn_tc_applicable(u32 n, u32 dim, int kind, u32 k, const f32* x);
void knn_tc(tt_ctx* c, const f32* x, u32 n, u32 k, u32* ids, f32* dists, bool defer);
void knn_tc_settle(tt_ctx* c);

namespace {
// Each point's cell: the nearest (squared L2; ties to the lower pivot) of P
// strided pivot points, the pivots' rows staged in shared memory.
__global__ void k_pivot_cell(const f32* __restrict__ x, u32 n, u32 dim, u32 P, u64* __restrict__ key,
                             u32* __restrict__ val) {
    pdl_wait();
    pdl_trigger();
    extern __shared__ f32 pv[];   // P x dim
    for (u32 t = threadIdx.x; t < P * dim; t += blockDim.x) pv[t] = x[(u64(t / dim) * n / P) * dim + t % dim];
    __syncthreads();
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const f32* xi = x + u64(i) * dim;
        u32 best = 0;
        f32 bd = INFINITY;
        for (u32 q = 0; q < P; ++q) {
            f32 s = 0.0f;
            for (u32 k = 0; k < dim; ++k) {
                const f32 u = xi[k] - pv[q * dim + k];
                s = fmaf(u, u, s);
            }
            if (s < bd) bd = s, best = q;
        }
        key[i] = best;
        val[i] = i;
    }
}
}  // namespace

// A query order for the exhaustive scan in which neighbouring points share
// warps: the points stably sorted by their cell among about n / 1536 pivots.
// (The Lp scan stops a candidate's sum early once it exceeds the query's
// bound; a warp waits for its slowest lane, so queries with similar
// neighbourhoods in one warp stop at similar points.)
static const u32* pivot_order(tt_ctx* c, const f32* x, u32 n, u32 dim) {
    const u32 P = std::max<u32>(2, std::min<u32>(128, n / 1536));
    u64* key = c->arena.get<u64>(S_TC_KEYS, n);
    u32* val = c->arena.get<u32>(S_TC_VALS, n);
    launch_pdl(k_pivot_cell, std::min<u32>(div_up(n, 256), 8 * u32(c->sms)), 256, sizeof(f32) * P * dim, c->stream, 
        x, n, dim, P, key, val);
    TT_LAUNCH("k_pivot_cell");
    ++c->launches;
    u64* kb = c->arena.get<u64>(S_SORT_A, n);
    u32* vb = c->arena.get<u32>(S_SORT_VA, n);
    return radix_sort<u32>(c, key, val, n, kb, vb, 32 - __builtin_clz(P - 1)) ? vb : val;
}

void knn_exact(tt_ctx* c, const f32* x, u32 n, u32 dim, int kind, f32 p, u32 k, u32* ids, f32* dists, bool defer) {
    if (k == 0 || n < 2) return;
    // L2 in R^32: the tensor-core Gram filter (tt_knn_tc.cu) unless the
    // context asks for the exhaustive scan; both give the same lists
    if (c->knn_mode != 1 && knn_tc_applicable(n, dim, kind, k, x) && (c->knn_mode == 2 || n >= 1024)) {
        knn_tc(c, x, n, k, ids, dists, defer);
        return;
    }
    u32* err = error_word(c);
    // (dimensions the scans refuse keep their own error: no order for them)
    const u32* order = kind == M_LP && n >= 4096 && dim <= scan::kMaxDim ? pivot_order(c, x, n, dim) : nullptr;
    if (k <= 16) scan_all(c, kind, x, n, dim, p, KnnOp<16>{ids, dists, k, order}, nullptr, err);
    else if (k <= 32) scan_all(c, kind, x, n, dim, p, KnnOp<32>{ids, dists, k, order}, nullptr, err);
    else invalid("gb300: exact kNN supports k <= 32");
    check_error_word(c, err);
}

// Symmetric union of the lists (graph.hpp:286-304): both directions of every
// list entry, sorted by (row, col), duplicates dropped. The weight of (i, j)
// is the list distance d(i, j), bit-identical to the reference's recomputed
// c(v, u) because every kernel is symmetric bit for bit.
u64 knn_graph(tt_ctx* c, const f32* x, u32 n, u32 dim, int kind, f32 p, const u32* ids, u32 k, u64* rp,
              u32** ci_out, f32** w_out) {
    const u64 m = 2 * u64(n) * k;
    u32* kid = const_cast<u32*>(ids);
    f32* kd = c->arena.get<f32>(S_KNN_D, u64(n) * k + 1);
    if (!ids) {
        kid = c->arena.get<u32>(S_KNN_I, u64(n) * k + 1);
        knn_exact(c, x, n, dim, kind, p, k, kid, kd, true);   // its status is read at the next round trip
        settle_finite(c);   // a pending check of the points: before the lists index anything
    } else {
        invalid("gb300: knn_graph from external lists is not supported; pass ids = NULL");
    }
    if (m) {
        // row-local path: count, scan, fill, per-row sort + dedupe
        const u32 gw = grid_for(u64(n) * 32, 256);
        u64* off = c->arena.get<u64>(S_MISC0, 2 * (u64(n) + 2));
        u64* ucnt = off + n + 2;
        u32* cur = c->arena.get<u32>(S_MISC1, u64(n) + 4);
        u32* ovf = cur + n;
        TT_CUDA(cudaMemsetAsync(off, 0, (u64(n) + 1) * sizeof(u64), c->stream));
        TT_CUDA(cudaMemsetAsync(cur, 0, (u64(n) + 1) * sizeof(u32), c->stream));
        launch_pdl(k_graph_deg, grid_for(u64(n) * k, 256), 256, 0, c->stream, kid, n, k,
                                                                        reinterpret_cast<unsigned long long*>(off));
        TT_LAUNCH("k_graph_deg");
        scan_exclusive<u64>(c, off, off, n, off + n);
        u32* col = c->arena.get<u32>(S_GRAPH_KEYS, 2 * m + 2);
        f32* cw = reinterpret_cast<f32*>(col + m + 1);
        u32* scol = c->arena.get<u32>(S_GRAPH_TMP, 2 * m + 2);
        f32* sw = reinterpret_cast<f32*>(scol + m + 1);
        launch_pdl(k_graph_fill, grid_for(u64(n) * k, 256), 256, 0, c->stream, kid, kd, n, k, off, cur, col, cw);
        TT_LAUNCH("k_graph_fill");
        u32* longs = c->arena.get<u32>(S_GRAPH_LONG, u64(n) + 1);
        TT_CUDA(cudaMemsetAsync(longs, 0, sizeof(u32), c->stream));
        launch_pdl(k_graph_rowsort, gw, 256, 0, c->stream, off, n, col, cw, scol, sw,
                                                    reinterpret_cast<unsigned long long*>(ucnt), ovf, longs);
        TT_LAUNCH("k_graph_rowsort");
        launch_pdl(k_graph_rowsort_long, std::min<u32>(n, 8 * u32(c->sms)), kLongThreads, 0, c->stream, 
            off, longs, col, cw, scol, sw, reinterpret_cast<unsigned long long*>(ucnt));
        TT_LAUNCH("k_graph_rowsort_long");
        c->launches += 4;
        // the row pointers from the distinct counts (meaningful only without
        // overflow); the CSR is emitted into buffers of the largest size
        // (2 n k entries) before the count and the overflow flag come back in
        // one round trip, so the emit runs while the host waits
        scan_exclusive<u64>(c, ucnt, rp, n, rp + n);
        u32* ci = c->arena.get<u32>(S_GRAPH_CI, m + 1);
        f32* w = c->arena.get<f32>(S_GRAPH_W, m + 1);
        launch_pdl(k_graph_emit, gw, 256, 0, c->stream, off, n, scol, sw, rp, ci, w, ovf);
        TT_LAUNCH("k_graph_emit");
        ++c->launches;
        u32 overflow = 0;
        u64 nnz = 0;
        TT_CUDA(cudaMemcpyAsync(&overflow, ovf, 4, cudaMemcpyDeviceToHost, c->stream));
        TT_CUDA(cudaMemcpyAsync(&nnz, rp + n, 8, cudaMemcpyDeviceToHost, c->stream));
        TT_CUDA(cudaStreamSynchronize(c->stream));
        knn_tc_settle(c);
        if (!overflow) {
            *ci_out = ci;
            *w_out = w;
            return nnz;
        }
    }
    // a row longer than kRowSortMax (a hub): one global sort of all 2 n k
    // directed entries by (row, column)
    u64* keys = c->arena.get<u64>(S_GRAPH_KEYS, m + 1);
    u32* vals = c->arena.get<u32>(S_GRAPH_TMP, m + 1);
    if (m) {
        k_knn_pairs<<<grid_for(u64(n) * k, 256), 256, 0, c->stream>>>(kid, kd, n, k, keys, vals);
        TT_LAUNCH("k_knn_pairs");
        ++c->launches;
    }
    radix_sort_inplace<u32>(c, keys, vals, m);
    u64* f = c->arena.get<u64>(S_MISC0, 2 * m + 4);
    u64* pos = f + m + 2;
    u64* tot = c->arena.get<u64>(S_COUNT, 4);
    u64 nnz = 0;
    if (m) {
        k_unique_flags<<<grid_for(m, 256), 256, 0, c->stream>>>(keys, m, f);
        scan_exclusive<u64>(c, f, pos, m, tot);
        TT_CUDA(cudaMemcpyAsync(&nnz, tot, 8, cudaMemcpyDeviceToHost, c->stream));
        TT_CUDA(cudaStreamSynchronize(c->stream));
        knn_tc_settle(c);
        ++c->launches;
    }
    u32* ci = c->arena.get<u32>(S_GRAPH_CI, nnz + 1);
    f32* w = c->arena.get<f32>(S_GRAPH_W, nnz + 1);
    u32* rows = c->arena.get<u32>(S_OUT3, nnz + 1);
    if (m) {
        k_unique_emit<<<grid_for(m, 256), 256, 0, c->stream>>>(keys, vals, m, f, pos, ci, w, rows);
        TT_LAUNCH("k_unique_emit");
        ++c->launches;
    }
    k_row_ptr<<<grid_for(nnz + 1, 256), 256, 0, c->stream>>>(rows, nnz, n, rp);
    TT_LAUNCH("k_row_ptr");
    ++c->launches;
    *ci_out = ci;
    *w_out = w;
    return nnz;
}

// radius_graph (graph.hpp:170-201): a counting scan, a scan of the counts
// into row pointers, and a filling scan that writes each row in increasing
// neighbour order (the order CsrGraph::from_rows sorts into).
u64 radius_graph(tt_ctx* c, const f32* x, u32 n, u32 dim, int kind, f32 p, f32 tau, u64* rp, u32** ci_out,
                 f32** w_out) {
    u64* cnt = c->arena.get<u64>(S_MISC0, u64(n) + 1);
    u64* tot = c->arena.get<u64>(S_COUNT, 4);
    u32* err = error_word(c);
    if (n) scan_all(c, kind, x, n, dim, p, RadiusCountOp{tau, cnt}, nullptr, err);
    scan_exclusive<u64>(c, cnt, rp, n, tot);
    TT_CUDA(cudaMemcpyAsync(rp + n, tot, 8, cudaMemcpyDeviceToDevice, c->stream));
    u64 nnz = 0;
    TT_CUDA(cudaMemcpyAsync(&nnz, tot, 8, cudaMemcpyDeviceToHost, c->stream));
    TT_CUDA(cudaStreamSynchronize(c->stream));
    u32* ci = c->arena.get<u32>(S_OUT1, nnz + 1);
    f32* w = c->arena.get<f32>(S_OUT2, nnz + 1);
    if (n) scan_all(c, kind, x, n, dim, p, RadiusFillOp{tau, rp, ci, w}, nullptr, err);
    check_error_word(c, err);
    *ci_out = ci;
    *w_out = w;
    return nnz;
}

// One Borůvka proposal scan over the complete graph: near[i] receives point
// i's minimum (d, combinatorial index) edge to another component, as float
// bits of d << 32 | the other endpoint (~0 when every point shares i's).
void foreign_nearest(tt_ctx* c, const f32* x, u32 n, u32 dim, int kind, f32 p, const u32* comp,
                     unsigned long long* near, u32* err, const u32* qlist, const u32* nq) {
    scan_all(c, kind, x, n, dim, p, ForeignOp{comp, near, qlist, nq}, comp, err);
}

void check_device_error(tt_ctx* c, const u32* err) { check_error_word(c, err); }
u32* device_error_word(tt_ctx* c) { return error_word(c); }

}  // namespace tt
