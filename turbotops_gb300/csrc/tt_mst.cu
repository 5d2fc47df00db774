// tt_mst.cu — H0 of the complete-graph Rips filtration via Borůvka.
//
// Replaces mst::h0 (mst.hpp:25-99). The reference grows one Prim tree; the
// finite H0 deaths are the weights of a minimum spanning tree, and every MST
// of a graph has the same multiset of weights, so any MST gives the same
// sorted death list. Here each round proposes, for every component, its
// minimum outgoing edge under the strict order (d, combinatorial index):
// the all-pairs scan of tt_knn.cu finds each point's nearest point of
// another component, then two passes over the points take the component's
// minimum distance and, among its points at that distance, the minimum
// edge index (64-bit: any n). The proposals form a forest (only mutual
// proposals close 2-cycles, broken by component id); components merge, and
// after at most ceil(log2 n) rounds one tree remains. The deaths are then
// sorted by a radix sort on their float bits.
//
// Above kKnnMin points the rounds start from each point's K nearest
// neighbours (one exact kNN pass; the tensor-core filter for L2 in R^32):
// the first list entry in another component is the point's nearest foreign
// point (the list holds the K smallest (d, j) of all points), and a point
// whose whole list lies in its own component has no foreign edge shorter than
// its K-th distance. Such an interior point can only carry its component's
// minimum when that K-th distance does not exceed the best proposal of the
// component's other points, so only those interior points are scanned (a
// listed subset of queries) before the per-component minima are taken:
// every round's proposals are the same as with a scan of every point.
#include "tt_internal.cuh"

namespace tt {

void foreign_nearest(tt_ctx* c, const f32* x, u32 n, u32 dim, int kind, f32 p, const u32* comp,
                     unsigned long long* near, u32* err, const u32* qlist = nullptr, const u32* nq = nullptr);
void check_device_error(tt_ctx* c, const u32* err);
u32* device_error_word(tt_ctx* c);

namespace {

constexpr u32 kNoD = 0xffffffffu;   // no proposal (above every float's bits)
constexpr u32 kKnnK = 16;           // neighbours a point keeps for the rounds
constexpr u32 kKnnMin = 4096;       // fewer points: every round scans every point

// From each point's list (ascending (d, id), K entries): the first entry in
// another component is its proposal, d bits << 32 | j; with none, near[i] =
// ~0 and kb[i] = the K-th entry's distance bits (a lower bound on every
// foreign edge of i).
__global__ void k_mst_knn_near(const u32* __restrict__ ids, const f32* __restrict__ dists, u32 K,
                               const u32* __restrict__ comp, unsigned long long* __restrict__ near,
                               u32* __restrict__ kb, u32 n) {
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const u32 ci = comp[i];
        u64 key = ~0ull;
        for (u32 t = 0; t < K; ++t) {
            const u32 j = ids[u64(i) * K + t];
            if (comp[j] != ci) {
                key = (u64(__float_as_uint(dists[u64(i) * K + t])) << 32) | j;
                break;
            }
        }
        near[i] = key;
        kb[i] = __float_as_uint(dists[u64(i) * K + K - 1]);
    }
}

// Interior points (no proposal from the list) whose K-th distance does not
// exceed their component's best proposal so far: listed for the scan.
__global__ void k_mst_flag(const unsigned long long* __restrict__ near, const u32* __restrict__ kb,
                           const u32* __restrict__ comp, const u32* __restrict__ bd, u32* __restrict__ qlist,
                           u32* __restrict__ nq, u32 n) {
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (near[i] == ~0ull && kb[i] <= bd[comp[i]]) qlist[atomicAdd(nq, 1u)] = i;
}

__global__ void k_mst_init(u32* __restrict__ comp, u32* __restrict__ parent, u32* __restrict__ bd,
                           u64* __restrict__ bi, u32 n) {
    for (u32 v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        comp[v] = v;
        parent[v] = v;
        bd[v] = kNoD;
        bi[v] = ~0ull;
    }
}

// Per component: the smallest distance bits among its points' proposals ...
__global__ void k_mst_min_d(const u32* __restrict__ comp, const unsigned long long* __restrict__ near,
                            u32* __restrict__ bd, u32 n) {
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const u64 k = near[i];
        if (k != ~0ull) atomicMin(&bd[comp[i]], u32(k >> 32));
    }
}

// ... and the smallest edge index among the proposals at that distance.
__global__ void k_mst_min_idx(const u32* __restrict__ comp, const unsigned long long* __restrict__ near,
                              const u32* __restrict__ bd, unsigned long long* __restrict__ bi, u32 n) {
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const u64 k = near[i];
        const u32 c = comp[i];
        if (k != ~0ull && u32(k >> 32) == bd[c]) atomicMin(&bi[c], (unsigned long long)edge_idx(i, u32(k)));
    }
}

__global__ void k_mst_hook(const u32* __restrict__ comp, const u32* __restrict__ bd, const u64* __restrict__ bi,
                           u32* __restrict__ parent, u32 n, f32* __restrict__ deaths, u32* __restrict__ cnt) {
    for (u32 c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        if (comp[c] != c || bd[c] == kNoD) continue;
        const u64 idx = bi[c];
        u32 a, b;
        decode_edge(idx, a, b);
        const u32 o = comp[a] == c ? comp[b] : comp[a];
        if (bi[o] == idx && c < o) continue;   // mutual: o hooks and records
        parent[c] = o;
        deaths[atomicAdd(cnt, 1u)] = __uint_as_float(bd[c]);
    }
}

__global__ void k_mst_flatten(const u32* __restrict__ parent, u32* __restrict__ comp, u32* __restrict__ bd,
                              u64* __restrict__ bi, u32 n) {
    for (u32 v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        u32 r = parent[v];
        for (u32 s = 0; parent[r] != r && s < n; ++s) r = parent[r];
        comp[v] = r;
        bd[v] = kNoD;
        bi[v] = ~0ull;
    }
}

__global__ void k_float_keys(const f32* __restrict__ d, u32 m, u64* __restrict__ keys) {
    for (u32 e = blockIdx.x * blockDim.x + threadIdx.x; e < m; e += gridDim.x * blockDim.x)
        keys[e] = __float_as_uint(d[e]);
}

__global__ void k_keys_float(const u64* __restrict__ keys, u32 m, f32* __restrict__ d) {
    for (u32 e = blockIdx.x * blockDim.x + threadIdx.x; e < m; e += gridDim.x * blockDim.x)
        d[e] = __uint_as_float(u32(keys[e]));
}

inline u32 grid_for(u64 work) { return u32(std::max<u64>(1, std::min<u64>((work + 255) / 256, 64ull * kSMs))); }

}  // namespace

// Sorted MST weights (n - 1 of them) into deaths (device). Returns n - 1.
u64 mst_deaths(tt_ctx* c, const f32* x, u32 n, u32 dim, int kind, f32 p, f32* deaths) {
    if (n < 2) return 0;
    u32* comp = c->arena.get<u32>(S_UF_PARENT, 2 * u64(n) + 2);
    u32* parent = comp + n + 1;
    unsigned long long* near = c->arena.get<unsigned long long>(S_UF_BEST, n + 1);
    u64* bi = c->arena.get<u64>(S_UF_WORK, n + 1);
    u32* bd = c->arena.get<u32>(S_UF_WORK2, n + 1);
    // the lists first (the kNN stage's own scratch is free again after it)
    const bool lists = n >= kKnnMin;
    const u32 K = std::min<u32>(kKnnK, n - 1);
    u32* kid = nullptr;
    f32* kd = nullptr;
    if (lists) {
        kid = c->arena.get<u32>(S_KNN_I, u64(n) * K + 1);
        kd = c->arena.get<f32>(S_KNN_D, u64(n) * K + 1);
        knn_exact(c, x, n, dim, kind, p, K, kid, kd, false);
        settle_finite(c);   // a pending check of the points: a NaN leaves a list short
    }
    u32* kb = lists ? c->arena.get<u32>(S_MST_KB, n + 1) : nullptr;
    u32* qlist = lists ? c->arena.get<u32>(S_MST_Q, n + 2) : nullptr;
    u32* nq = lists ? qlist + n + 1 : nullptr;
    u32* cnt = c->arena.get<u32>(S_MISC1, 4);
    u32* err = device_error_word(c);
    k_mst_init<<<grid_for(n), 256, 0, c->stream>>>(comp, parent, bd, bi, n);
    TT_CUDA(cudaMemsetAsync(cnt, 0, sizeof(u32), c->stream));
    c->launches += 1;
    u32 done = 0;
    for (int round = 0; round < 40 && done < n - 1; ++round) {
        if (lists) {
            k_mst_knn_near<<<grid_for(n), 256, 0, c->stream>>>(kid, kd, K, comp, near, kb, n);
            k_mst_min_d<<<grid_for(n), 256, 0, c->stream>>>(comp, near, bd, n);
            TT_CUDA(cudaMemsetAsync(nq, 0, sizeof(u32), c->stream));
            k_mst_flag<<<grid_for(n), 256, 0, c->stream>>>(near, kb, comp, bd, qlist, nq, n);
            c->launches += 3;
            foreign_nearest(c, x, n, dim, kind, p, comp, near, err, qlist, nq);
        } else {
            foreign_nearest(c, x, n, dim, kind, p, comp, near, err);
        }
        k_mst_min_d<<<grid_for(n), 256, 0, c->stream>>>(comp, near, bd, n);
        k_mst_min_idx<<<grid_for(n), 256, 0, c->stream>>>(comp, near, bd, reinterpret_cast<unsigned long long*>(bi),
                                                          n);
        k_mst_hook<<<grid_for(n), 256, 0, c->stream>>>(comp, bd, bi, parent, n, deaths, cnt);
        k_mst_flatten<<<grid_for(n), 256, 0, c->stream>>>(parent, comp, bd, bi, n);
        TT_LAUNCH("mst round");
        c->launches += 4;
        u32 h = 0;
        TT_CUDA(cudaMemcpyAsync(&h, cnt, 4, cudaMemcpyDeviceToHost, c->stream));
        TT_CUDA(cudaStreamSynchronize(c->stream));
        if (h == done) break;   // no progress: cannot happen on a connected complete graph
        done = h;
    }
    check_device_error(c, err);
    if (done != n - 1) throw Error(TT_ERR_INTERNAL, "gb300: Boruvka did not span the cloud");
    u64* keys = c->arena.get<u64>(S_EDGE_KEYS, n);
    k_float_keys<<<grid_for(n - 1), 256, 0, c->stream>>>(deaths, n - 1, keys);
    radix_sort_inplace<u32>(c, keys, nullptr, n - 1);
    k_keys_float<<<grid_for(n - 1), 256, 0, c->stream>>>(keys, n - 1, deaths);
    TT_LAUNCH("mst sort");
    c->launches += 2;
    return n - 1;
}

}  // namespace tt
