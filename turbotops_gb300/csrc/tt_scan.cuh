// tt_scan.cuh — the tiled all-pairs scanner shared by the kNN, radius-graph
// and Borůvka kernels (tt_knn.cu and tt_mst.cu say what each visitor
// replaces in the reference).
//
// A CTA owns kQ queries (one per thread, the query's coordinates in
// registers) and streams every candidate point through shared memory in tiles
// of kCB points. Full tiles arrive by bulk TMA copies (cp.async.bulk +
// mbarrier, double-buffered) when a point row is a multiple of 16 bytes;
// otherwise the CTA loads them cooperatively. Candidates are visited in
// increasing id order, which is what makes the (distance, id) tie rule a
// strict-less test on the distance. DIM = 0 is the runtime-dimension variant
// (query read through L1) for dimensions without a specialisation.
//
// Each metric kind is instantiated in its own translation unit
// (tt_scan_<kind>.cu) so the build compiles them in parallel.
#pragma once
#include <type_traits>

#include "tt_internal.cuh"
#include "tt_metric.cuh"
#include "tt_tma.cuh"

namespace tt {
namespace scan {

constexpr int kQ = 128;    // queries (threads) per CTA
constexpr int kCB = 128;   // candidates per shared-memory tile
constexpr u32 kMaxDim = 64;

template <int DIM>
struct RegRow {
    const f32 (&q)[DIM];
    __device__ __forceinline__ f32 operator()(u32 k) const { return q[k]; }
};

// --------------------------------------------------------------------------
// Per-query visitors.
// --------------------------------------------------------------------------
// Top-K by (distance, id) in registers (knn_query's heap, graph.hpp:123-166).
// With qlist, the CTAs take their queries in that order (a permutation of the
// points): the lists are the same, since every comparison is on (distance,
// id), and queries that lie close together share warps.
template <int K>
struct KnnOp {
    u32* ids;
    f32* dists;
    u32 k;
    const u32* qlist = nullptr;
    struct State {
        f32 d[K];
        u32 j[K];
        f32 thr_s;   // sq_bound of the current K-th distance
    };
    __device__ __forceinline__ void init(State& s, u32) const {
#pragma unroll
        for (int t = 0; t < K; ++t) {
            s.d[t] = INFINITY;
            s.j[t] = 0xffffffffu;
        }
        s.thr_s = INFINITY;
    }
    // L2 fast path: the squared sum decides most candidates; only those that
    // can still enter the list take the IEEE square root.
    __device__ __forceinline__ void visit_sq(State& s, u32 i, u32 j, f32 sq, const u32*) const {
        if (j == i || sq > s.thr_s) return;
        visit(s, i, j, __fsqrt_rn(sq), nullptr);
        s.thr_s = sq_bound(s.d[K - 1]);
    }
    // Largest distance that can still enter the list (Lp pre-test).
    __device__ __forceinline__ f32 bound(const State& s) const { return s.d[K - 1]; }
    __device__ __forceinline__ static bool lt(f32 d, u32 j, f32 e, u32 i) { return d < e || (d == e && j < i); }
    __device__ __forceinline__ void visit(State& s, u32 i, u32 j, f32 d, const u32*) const {
        if (j == i || !lt(d, j, s.d[K - 1], s.j[K - 1])) return;
        bool placed = false;
#pragma unroll
        for (int t = K - 1; t >= 1; --t) {
            if (!placed) {
                if (lt(d, j, s.d[t - 1], s.j[t - 1])) {
                    s.d[t] = s.d[t - 1];
                    s.j[t] = s.j[t - 1];
                } else {
                    s.d[t] = d;
                    s.j[t] = j;
                    placed = true;
                }
            }
        }
        if (!placed) {
            s.d[0] = d;
            s.j[0] = j;
        }
    }
    __device__ __forceinline__ void finish(const State& s, u32 i) const {
#pragma unroll
        for (int t = 0; t < K; ++t)
            if (t < int(k)) {
                ids[u64(i) * k + t] = s.j[t];
                if (dists) dists[u64(i) * k + t] = s.d[t];
            }
    }
};

struct RadiusCountOp {
    f32 tau;
    u64* cnt;
    struct State {
        u64 c;
    };
    __device__ __forceinline__ void init(State& s, u32) const { s.c = 0; }
    __device__ __forceinline__ f32 bound(const State&) const { return tau; }
    __device__ __forceinline__ void visit(State& s, u32 i, u32 j, f32 d, const u32*) const {
        s.c += (j != i && d <= tau);
    }
    __device__ __forceinline__ void finish(const State& s, u32 i) const { cnt[i] = s.c; }
};

struct RadiusFillOp {
    f32 tau;
    const u64* rp;
    u32* ci;
    f32* w;
    struct State {
        u64 o;
    };
    __device__ __forceinline__ void init(State& s, u32 i) const { s.o = rp[i]; }
    __device__ __forceinline__ f32 bound(const State&) const { return tau; }
    __device__ __forceinline__ void visit(State& s, u32 i, u32 j, f32 d, const u32*) const {
        if (j != i && d <= tau) {
            ci[s.o] = j;
            w[s.o] = d;
            ++s.o;
        }
    }
    __device__ __forceinline__ void finish(const State&, u32) const {}
};

// Each point's nearest point of another component under the strict edge
// order (d, combinatorial index): for a fixed point i the index of edge
// (i, j) grows with j, so the per-point minimum of (d, j) is the minimum of
// (d, index) over i's edges. near[i] = float bits of d << 32 | j (~0: none);
// the Borůvka round (tt_mst.cu) reduces these per component. With qlist,
// only the *nq points it lists are queries (the scan's grid covers n; the
// CTAs past *nq return at once) and the other points' near[] stay as they are.
struct ForeignOp {
    const u32* comp;
    unsigned long long* near;   // per point
    const u32* qlist = nullptr;
    const u32* nq = nullptr;
    struct State {
        u64 key;
        u32 c;
        f32 thr_s;
    };
    __device__ __forceinline__ void init(State& s, u32 i) const {
        s.key = ~0ull;
        s.c = comp[i];
        s.thr_s = INFINITY;
    }
    __device__ __forceinline__ void visit_sq(State& s, u32 i, u32 j, f32 sq, const u32* tcomp) const {
        if (tcomp[0] == s.c || sq > s.thr_s) return;
        visit(s, i, j, __fsqrt_rn(sq), tcomp);
        s.thr_s = sq_bound(__uint_as_float(u32(s.key >> 32)));
    }
    // The current proposal's distance (NaN while there is none: never skips).
    __device__ __forceinline__ f32 bound(const State& s) const {
        return __uint_as_float(u32(s.key >> 32));
    }
    __device__ __forceinline__ void visit(State& s, u32, u32 j, f32 d, const u32* tcomp) const {
        if (tcomp[0] == s.c) return;
        const u64 key = (u64(__float_as_uint(d)) << 32) | j;
        if (key < s.key) s.key = key;
    }
    __device__ __forceinline__ void finish(const State& s, u32 i) const { near[i] = s.key; }
};

template <typename Op>
struct NeedsComp : std::false_type {};
// Visitors whose queries may come from a list.
template <typename Op>
struct ListedQueries : std::false_type {};
template <int K>
struct ListedQueries<KnnOp<K>> : std::true_type {};
template <>
struct NeedsComp<ForeignOp> : std::true_type {};

// Visitors that accept the L2 squared sum (visit_sq) before the root.
template <typename Op>
struct TakesSq : std::false_type {};
template <int K>
struct TakesSq<KnnOp<K>> : std::true_type {};
template <>
struct TakesSq<ForeignOp> : std::true_type {};

// --------------------------------------------------------------------------
// The scanner (compiled only in the tt_scan_<kind>.cu translation units).
// --------------------------------------------------------------------------
#ifdef TT_SCAN_IMPL
template <int KIND, int DIM, typename Op>
__global__ void __launch_bounds__(kQ)
k_scan(const f32* __restrict__ x, u32 n, u32 dim_rt, f32 p, Op op, const u32* __restrict__ comp,
       u32* __restrict__ err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr bool kRt = DIM == 0;
    const u32 dim = kRt ? dim_rt : u32(DIM);
    f32* tiles = reinterpret_cast<f32*>(smem_raw);                 // [2][kCB * dim]
    u32* tcomp = reinterpret_cast<u32*>(tiles + 2 * kCB * dim);    // [2][kCB]
    __shared__ __align__(8) u64 bar[2];
    const u32 tid = threadIdx.x;
    u32 i = blockIdx.x * kQ + tid;
    if constexpr (std::is_same<Op, ForeignOp>::value) {
        if (op.qlist) {   // a listed subset of the points (block-uniform exit past its end)
            const u32 nq = *op.nq;
            if (blockIdx.x * kQ >= nq) return;
            i = i < nq ? op.qlist[i] : n;
        }
    } else if constexpr (ListedQueries<Op>::value) {
        if (op.qlist && i < n) i = op.qlist[i];   // every point, in the list's order
    }
    const bool active = i < n;
    constexpr int QN = kRt ? 1 : DIM;
    f32 q[QN];
    if (!kRt) {
#pragma unroll
        for (int k = 0; k < QN; ++k) q[k] = active ? x[u64(i) * QN + k] : 0.0f;
    }
    const f32* qg = x + u64(active ? i : 0) * dim;
    typename Op::State st;
    if (active) op.init(st, i);

    const u32 ntiles = (n + kCB - 1) / kCB;
    const bool bulk = (dim * 4) % 16 == 0 && (reinterpret_cast<uintptr_t>(x) & 15) == 0;
    constexpr bool kComp = NeedsComp<Op>::value;
    auto issue = [&](u32 t, int buf) {
        const u32 j0 = t * kCB, rows = min(u32(kCB), n - j0);
        const u32 bytes = rows * dim * 4;
        mbar_expect_tx(&bar[buf], bytes);
        bulk_g2s(tiles + buf * kCB * dim, x + u64(j0) * dim, bytes, &bar[buf]);
    };
    if (bulk) {
        if (tid == 0) {
            mbar_init(&bar[0], 1);
            mbar_init(&bar[1], 1);
            fence_mbar_init();
        }
        __syncthreads();
        if (tid == 0) {
            issue(0, 0);
            if (ntiles > 1) issue(1, 1);
        }
    }
    for (u32 t = 0; t < ntiles; ++t) {
        const int buf = bulk ? int(t & 1) : 0;
        const u32 j0 = t * kCB, rows = min(u32(kCB), n - j0);
        f32* tile = tiles + buf * kCB * dim;
        u32* tc = tcomp + buf * kCB;
        if (kComp)
            for (u32 r = tid; r < rows; r += kQ) tc[r] = comp[j0 + r];
        if (bulk) {
            mbar_wait(&bar[buf], (t >> 1) & 1, err);
        } else {
            for (u32 e = tid; e < rows * dim; e += kQ) tile[e] = x[u64(j0) * dim + e];
        }
        __syncthreads();
        if (active) {
            if constexpr (KIND == M_LP) {
                // Lp: the exact root (glibc powf replay, double precision)
                // only for candidates a float lower bound cannot reject
                for (u32 r = 0; r < rows; ++r) {
                    f32 M, sum;
                    const f32 bd = op.bound(st);
                    const bool within = kRt ? lp_parts_within(Row{qg}, Row{tile + r * dim}, dim, p, bd, M, sum)
                                            : lp_parts_within(RegRow<QN>{q}, Row{tile + r * QN}, QN, p, bd, M, sum);
                    if (!within || lp_root_lower(M, sum, p) > bd) continue;
                    op.visit(st, i, j0 + r, lp_root(M, sum, p), kComp ? tc + r : nullptr);
                }
            } else if (kRt) {
                for (u32 r = 0; r < rows; ++r) {
                    const f32 d = metric_dist(KIND, p, Row{qg}, Row{tile + r * dim}, dim);
                    op.visit(st, i, j0 + r, d, kComp ? tc + r : nullptr);
                }
            } else if constexpr (KIND == M_L2 && TakesSq<Op>::value && QN % 4 == 0) {
                // candidate row through 128-bit shared loads, squared sum
                // first (sq_bound pre-test), root only for survivors
#pragma unroll 2
                for (u32 r = 0; r < rows; ++r) {
                    f32 cr[QN];
                    const float4* c4 = reinterpret_cast<const float4*>(tile + r * QN);
#pragma unroll
                    for (int v = 0; v < QN / 4; ++v) {
                        const float4 t4 = c4[v];
                        cr[4 * v] = t4.x;
                        cr[4 * v + 1] = t4.y;
                        cr[4 * v + 2] = t4.z;
                        cr[4 * v + 3] = t4.w;
                    }
                    const f32 sq = l2_sq_acc(RegRow<QN>{q}, RegRow<QN>{cr}, QN);
                    op.visit_sq(st, i, j0 + r, sq, kComp ? tc + r : nullptr);
                }
            } else {
#pragma unroll 2
                for (u32 r = 0; r < rows; ++r) {
                    const f32 d = metric_dist(KIND, p, RegRow<QN>{q}, Row{tile + r * QN}, QN);
                    op.visit(st, i, j0 + r, d, kComp ? tc + r : nullptr);
                }
            }
        }
        __syncthreads();
        if (bulk && tid == 0 && t + 2 < ntiles) issue(t + 2, buf);
    }
    if (active) op.finish(st, i);
}

template <int KIND, int DIM, typename Op>
void launch(tt_ctx* c, const f32* x, u32 n, u32 dim, f32 p, const Op& op, const u32* comp, u32* err) {
    const size_t smem = size_t(2) * kCB * dim * 4 + 2 * kCB * 4;
    auto kfn = k_scan<KIND, DIM, Op>;
    TT_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    kfn<<<div_up(n, kQ), kQ, smem, c->stream>>>(x, n, dim, p, op, comp, err);
    TT_LAUNCH("k_scan");
    ++c->launches;
}

// One metric kind, every dimension specialisation.
template <int KIND, typename Op>
void scan_kind(tt_ctx* c, const f32* x, u32 n, u32 dim, f32 p, const Op& op, const u32* comp, u32* err) {
    if (dim == 0 || dim > kMaxDim) invalid("gb300: all-pairs scans support 1 <= dim <= 64");
    switch (dim) {
        case 2: launch<KIND, 2>(c, x, n, dim, p, op, comp, err); break;
        case 3: launch<KIND, 3>(c, x, n, dim, p, op, comp, err); break;
        case 4: launch<KIND, 4>(c, x, n, dim, p, op, comp, err); break;
        case 8: launch<KIND, 8>(c, x, n, dim, p, op, comp, err); break;
        case 16: launch<KIND, 16>(c, x, n, dim, p, op, comp, err); break;
        case 32: launch<KIND, 32>(c, x, n, dim, p, op, comp, err); break;
        default: launch<KIND, 0>(c, x, n, dim, p, op, comp, err); break;
    }
}

#define TT_SCAN_INSTANTIATE(KIND)                                                                             \
    template void scan_kind<KIND, KnnOp<16>>(tt_ctx*, const f32*, u32, u32, f32, const KnnOp<16>&, const u32*, \
                                             u32*);                                                           \
    template void scan_kind<KIND, KnnOp<32>>(tt_ctx*, const f32*, u32, u32, f32, const KnnOp<32>&, const u32*, \
                                             u32*);                                                           \
    template void scan_kind<KIND, RadiusCountOp>(tt_ctx*, const f32*, u32, u32, f32, const RadiusCountOp&,     \
                                                 const u32*, u32*);                                           \
    template void scan_kind<KIND, RadiusFillOp>(tt_ctx*, const f32*, u32, u32, f32, const RadiusFillOp&,       \
                                                const u32*, u32*);                                            \
    template void scan_kind<KIND, ForeignOp>(tt_ctx*, const f32*, u32, u32, f32, const ForeignOp&, const u32*, \
                                             u32*);
#endif  // TT_SCAN_IMPL

// Runtime dispatch over the metric kind (instantiations live in
// tt_scan_<kind>.cu).
template <int KIND, typename Op>
void scan_kind(tt_ctx* c, const f32* x, u32 n, u32 dim, f32 p, const Op& op, const u32* comp, u32* err);

template <typename Op>
void scan_all(tt_ctx* c, int kind, const f32* x, u32 n, u32 dim, f32 p, const Op& op, const u32* comp, u32* err) {
    switch (kind) {
        case M_L1: scan_kind<M_L1>(c, x, n, dim, p, op, comp, err); break;
        case M_L2: scan_kind<M_L2>(c, x, n, dim, p, op, comp, err); break;
        case M_LINF: scan_kind<M_LINF>(c, x, n, dim, p, op, comp, err); break;
        default: scan_kind<M_LP>(c, x, n, dim, p, op, comp, err); break;
    }
}

}  // namespace scan
}  // namespace tt
