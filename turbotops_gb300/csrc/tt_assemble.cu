// tt_assemble.cu — dimension-2 columns of the cohomology reducer on the GPU.
//
// Replaces rips.hpp Reducer::assemble(1) (:981-1023) over a dense complex:
// every kept edge s = (a > b) of diameter d_s contributes its cofacets
// t = (w > a > b), w > a, with diameter cd = max(d_s, D[a][w], D[b][w]) <=
// threshold (cofacets_full with all = false, :282-344). A cofacet is skipped
// when it is a pivot of the dimension-1 reduction (PivotMap lookup, :1001) or
// in a zero-apparent pair (zero_apparent_cofacet_v / zero_apparent_facet_v,
// :638-649, :1006-1007); the rest become columns, sorted in descending
// filtration order (:1019).
//
// Work mapping: one warp per edge. The 32 lanes take 32 apex candidates w
// at once (coalesced row segments of D[a] and D[b]) and test the threshold
// and pivot membership in parallel (open-addressing hash set of the pivots
// in device memory); each surviving triangle is then tested by the whole
// warp, whose lanes scan 32 candidate vertices per step of the descending
// cofacet search (zero_pivot_cofacet_v, :585-605). Columns are appended with
// one atomic per warp batch and radix-sorted by a descending key.
#include "tt_internal.cuh"

namespace tt {

namespace {

constexpr u32 NOV = 0xffffffffu;
constexpr u64 kEmpty = ~0ull;

__device__ __forceinline__ u64 hash64(u64 x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

__global__ void k_hash_insert(const u64* __restrict__ keys, u64 nk, u64* __restrict__ table, u64 mask) {
    for (u64 i = u64(blockIdx.x) * blockDim.x + threadIdx.x; i < nk; i += u64(gridDim.x) * blockDim.x) {
        const u64 k = keys[i];
        for (u64 s = hash64(k) & mask, probe = 0; probe <= mask; s = (s + 1) & mask, ++probe) {
            const unsigned long long prev = atomicCAS((unsigned long long*)&table[s], kEmpty, k);
            if (prev == kEmpty || prev == k) break;
        }
    }
}

__device__ __forceinline__ bool hash_contains(const u64* __restrict__ table, u64 mask, u64 k) {
    for (u64 s = hash64(k) & mask, probe = 0; probe <= mask; s = (s + 1) & mask, ++probe) {
        const u64 v = table[s];
        if (v == k) return true;
        if (v == kEmpty) return false;
    }
    return false;
}

// Largest v outside {x0..x(k-1)} with D[x_i][v] <= cap for every i (the
// first cofacet in descending index order); warp-cooperative, NOV if none.
template <int KR>
__device__ __forceinline__ u32 warp_top_cofacet(const f32* __restrict__ mat, u32 n, const u32 (&x)[KR], f32 cap) {
    const int lane = threadIdx.x & 31;
    for (int64_t hi = n; hi > 0; hi -= 32) {
        const int64_t v = hi - 32 + lane;
        bool ok = v >= 0;
        if (ok) {
#pragma unroll
            for (int i = 0; i < KR; ++i) ok = ok && u32(v) != x[i] && mat[u64(x[i]) * n + v] <= cap;
        }
        const u32 bal = __ballot_sync(0xffffffffu, ok);
        if (bal) return u32(hi - 32 + (31 - __clz(bal)));
    }
    return NOV;
}

__device__ __forceinline__ f32 D(const f32* __restrict__ mat, u32 n, u32 i, u32 j) {
    return i == j ? 0.0f : mat[u64(i) * n + j];
}

__device__ __forceinline__ u64 tet_idx(u32 a, u32 b, u32 c, u32 d) {   // a > b > c > d
    return u64(a) * (a - 1) * (a - 2) * (a - 3) / 24 + u64(b) * (b - 1) * (b - 2) / 6 + u64(c) * (c - 1) / 2 + d;
}

// zero_apparent_cofacet_v ∨ zero_apparent_facet_v for the triangle
// (c0 > c1 > c2) of diameter cd and index idx (rips.hpp:638-649).
__device__ bool triangle_apparent(const f32* __restrict__ mat, u32 n, u32 c0, u32 c1, u32 c2, f32 cd, u64 idx) {
    // zero_apparent_cofacet_v: the first cofacet of diameter cd, then its
    // first facet in ascending order must be this triangle.
    {
        const u32 x[3] = {c0, c1, c2};
        const u32 v = warp_top_cofacet<3>(mat, n, x, cd);
        if (v != NOV) {
            u32 t[4] = {c0, c1, c2, v};
            // sort descending (v is the only unsorted element)
#pragma unroll
            for (int i = 3; i > 0; --i)
                if (t[i] > t[i - 1]) { const u32 q = t[i]; t[i] = t[i - 1]; t[i - 1] = q; }
            // facet j (vertex j removed) has diameter cd iff an edge of length
            // cd avoids j; facets never exceed cd (zero_pivot_facet_v :609-636)
            const f32 e01 = D(mat, n, t[0], t[1]), e02 = D(mat, n, t[0], t[2]), e03 = D(mat, n, t[0], t[3]);
            const f32 e12 = D(mat, n, t[1], t[2]), e13 = D(mat, n, t[1], t[3]), e23 = D(mat, n, t[2], t[3]);
            u64 f = kNone;
            if (e12 == cd || e13 == cd || e23 == cd) f = tri_idx(t[1], t[2], t[3]);
            else if (e02 == cd || e03 == cd || e23 == cd) f = tri_idx(t[0], t[2], t[3]);
            else if (e01 == cd || e03 == cd || e13 == cd) f = tri_idx(t[0], t[1], t[3]);
            else if (e01 == cd || e02 == cd || e12 == cd) f = tri_idx(t[0], t[1], t[2]);
            if (f == idx) return true;
        }
    }
    // zero_apparent_facet_v: the first facet of diameter cd, then its first
    // cofacet in descending order must be this triangle.
    {
        u32 f0, f1;
        if (D(mat, n, c1, c2) == cd) { f0 = c1; f1 = c2; }
        else if (D(mat, n, c0, c2) == cd) { f0 = c0; f1 = c2; }
        else if (D(mat, n, c0, c1) == cd) { f0 = c0; f1 = c1; }
        else return false;
        const u32 x[2] = {f0, f1};
        const u32 w = warp_top_cofacet<2>(mat, n, x, cd);
        if (w == NOV) return false;
        u32 g0 = f0, g1 = f1, g2 = w;
        sort3(g0, g1, g2);
        return g0 == c0 && g1 == c1 && g2 == c2;
    }
}

// Columns as descending-order keys: (0x7fffffff - d bits) << 33 | idx, so an
// ascending sort gives d descending, index ascending (sort_desc, :680-682).
__global__ void __launch_bounds__(256)
k_assemble(const f32* __restrict__ mat, u32 n, f32 thr, const u64* __restrict__ keys, u64 m,
           const u64* __restrict__ piv, u64 pmask, int have_piv, u64* __restrict__ out, u64 cap,
           unsigned long long* __restrict__ counters) {
    const int lane = threadIdx.x & 31;
    const u64 warps = (u64(gridDim.x) * blockDim.x) >> 5;
    unsigned long long skipped = 0;
    for (u64 e = (u64(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; e < m; e += warps) {
        const u64 key = keys[e];
        const f32 ds = key_d(key);
        u32 a, b;
        decode_edge(key_idx(key), a, b);
        const f32* ra = mat + u64(a) * n;
        const f32* rb = mat + u64(b) * n;
        for (u32 w0 = a + 1; w0 < n; w0 += 32) {
            const u32 w = w0 + lane;
            f32 cd = 0.0f;
            bool cand = false;
            u64 idx = 0;
            if (w < n) {
                cd = fmaxf(ds, fmaxf(ra[w], rb[w]));
                cand = cd <= thr;
                if (cand) {
                    idx = tri_idx(w, a, b);
                    if (have_piv && hash_contains(piv, pmask, idx)) cand = false;
                }
            }
            u32 bal = __ballot_sync(0xffffffffu, cand);
            u32 keep = 0;
            while (bal) {
                const int src = __ffs(bal) - 1;
                bal &= bal - 1;
                const u32 tw = __shfl_sync(0xffffffffu, w, src);
                const f32 tcd = __shfl_sync(0xffffffffu, cd, src);
                const u64 tidx = __shfl_sync(0xffffffffu, idx, src);
                const bool app = triangle_apparent(mat, n, tw, a, b, tcd, tidx);
                if (app) ++skipped;
                else keep |= 1u << src;
            }
            if (keep) {
                unsigned long long base = 0;
                if (lane == 0) base = atomicAdd(&counters[0], (unsigned long long)__popc(keep));
                base = __shfl_sync(0xffffffffu, base, 0);
                if ((keep >> lane) & 1u) {
                    const u64 o = base + __popc(keep & ((1u << lane) - 1));
                    if (o < cap) out[o] = (u64(0x7fffffffu - __float_as_uint(cd)) << kIdxBits) | idx;
                }
            }
        }
    }
    // lanes of a warp count the same skips: lane 0 reports them
    if (lane == 0 && skipped) atomicAdd(&counters[1], skipped);
}

__global__ void k_split_columns(const u64* __restrict__ k, u64 c, u64* __restrict__ idx, f32* __restrict__ d) {
    for (u64 e = u64(blockIdx.x) * blockDim.x + threadIdx.x; e < c; e += u64(gridDim.x) * blockDim.x) {
        idx[e] = k[e] & kIdxMask;
        d[e] = __uint_as_float(0x7fffffffu - u32(k[e] >> kIdxBits));
    }
}

inline u32 grid_for(u64 work, u32 per_block) {
    const u64 g = (work + per_block - 1) / per_block;
    return u32(std::max<u64>(1, std::min<u64>(g, 32ull * kSMs)));
}

}  // namespace

// Columns of dimension 2 from the sorted kept edges `keys` (Ripser keys, m of
// them) and the dimension-1 pivots. Returns the column count; *cidx / *cd
// point at context-owned device arrays in descending filtration order.
u64 assemble2(tt_ctx* c, const Complex& cx, const u64* keys, u64 m, const u64* piv, u64 npiv, u64** cidx_out,
              f32** cd_out, u64* napp) {
    if (!cx.mat) invalid("gb300: assemble supports the dense complex");
    const u32 n = cx.n;
    if (n >= 3 && u64(n) * (n - 1) * (n - 2) / 6 >= (1ull << kIdxBits))
        invalid("gb300: assemble supports C(n, 3) < 2^33 (n <= 3740)");
    // pivot hash set (load <= 1/2)
    u64 slots = 16;
    while (slots < 2 * npiv + 2) slots <<= 1;
    u64* table = c->arena.get<u64>(S_ASM0, slots);
    TT_CUDA(cudaMemsetAsync(table, 0xff, slots * sizeof(u64), c->stream));
    if (npiv) {
        k_hash_insert<<<grid_for(npiv, 256), 256, 0, c->stream>>>(piv, npiv, table, slots - 1);
        TT_LAUNCH("k_hash_insert");
        ++c->launches;
    }
    unsigned long long* ctr = c->arena.get<unsigned long long>(S_ASM1, 2);
    u64 cap = std::max<u64>(1 << 20, 2 * m);
    unsigned long long h[2] = {0, 0};
    for (int attempt = 0; attempt < 2; ++attempt) {
        u64* out = c->arena.get<u64>(S_ASM2, cap);
        TT_CUDA(cudaMemsetAsync(ctr, 0, 2 * sizeof(unsigned long long), c->stream));
        if (m) {
            k_assemble<<<grid_for(m * 32, 256), 256, 0, c->stream>>>(cx.mat, n, cx.thr, keys, m, table, slots - 1,
                                                                     npiv > 0, out, cap, ctr);
            TT_LAUNCH("k_assemble");
            ++c->launches;
        }
        TT_CUDA(cudaMemcpyAsync(h, ctr, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
        TT_CUDA(cudaStreamSynchronize(c->stream));
        if (h[0] <= cap) break;
        cap = h[0] + h[0] / 8 + 16;   // rerun once with room for every column
    }
    const u64 cols = h[0];
    u64* out = c->arena.get<u64>(S_ASM2, cap);
    radix_sort_inplace<u32>(c, out, nullptr, cols);
    u64* cidx = c->arena.get<u64>(S_ASM3, cols + 1);
    f32* cd = c->arena.get<f32>(S_ASM4, cols + 1);
    if (cols) {
        k_split_columns<<<grid_for(cols, 256), 256, 0, c->stream>>>(out, cols, cidx, cd);
        TT_LAUNCH("k_split_columns");
        ++c->launches;
    }
    *cidx_out = cidx;
    *cd_out = cd;
    if (napp) *napp = h[1];
    return cols;
}

}  // namespace tt
