// tt_dim0.cu — the dimension-0 stage of the cohomology reducer on the GPU.
//
// Replaces rips.hpp Reducer::dim0 (:685-870): the kept edges (d <= thr) are
// packed into Ripser-order keys and radix-sorted (the reference's bucket sort
// reproduces the plain (d asc, idx desc) order, :775-839, which is what the
// key order is); every edge gets its zero-apparent-cofacet test (:844-849,
// zero_apparent_cofacet_v :644-649); the spanning forest that the reference's
// serial union-find selects over the sorted edges (:850-866) is computed by
// Borůvka over the edge ranks — with distinct ranks the minimum spanning
// forest is unique, so the tree/non-tree split is the same edge for edge.
// H0 bars are the tree edges with d > 0 in sorted order; columns are the
// non-tree, non-apparent edges in descending order (:867).
//
// For each non-apparent edge the kernel also records the column-local part of
// the emergent-pair shortcut of compute_pairs (:903-928): the first cofacet in
// descending order with the edge's diameter, and whether that cofacet has a
// zero-apparent facet. Only the pivot lookup stays on the host.
//
// The same stage covers the sparse complex (rips.hpp SparseComplex :418-472):
// cofacets of an edge are the common neighbours of its endpoints, walked from
// the top of their sorted CSR rows.
#include "tt_internal.cuh"

namespace tt {

namespace {

constexpr u32 NOV = 0xffffffffu;   // no vertex

// --------------------------------------------------------------------------
// Dense complex (full n x n matrix).
// --------------------------------------------------------------------------
struct DenseCx {
    const f32* mat;
    u32 n;
    __device__ __forceinline__ f32 d(u32 i, u32 j) const { return i == j ? 0.0f : mat[u64(i) * n + j]; }
};

// Largest w not in {a, b} with D[a][w] <= cap and D[b][w] <= cap, scanning
// candidates downward 32 at a time (coalesced row segments); NOV if none.
// This is the first cofacet in descending index order (cofacets_full
// rips.hpp:282-344 with all = true).
__device__ __forceinline__ u32 warp_top_cofacet2(const DenseCx& cx, u32 a, u32 b, f32 cap) {
    const int lane = threadIdx.x & 31;
    const f32* ra = cx.mat + u64(a) * cx.n;
    const f32* rb = cx.mat + u64(b) * cx.n;
    for (int64_t hi = cx.n; hi > 0; hi -= 32) {
        const int64_t w = hi - 32 + lane;
        bool ok = false;
        if (w >= 0 && u32(w) != a && u32(w) != b) ok = ra[w] <= cap && rb[w] <= cap;
        const u32 bal = __ballot_sync(0xffffffffu, ok);
        if (bal) return u32(hi - 32 + (31 - __clz(bal)));
    }
    return NOV;
}

// First facet of triangle (c0 > c1 > c2) in ascending index order with length
// d (zero_pivot_facet_v rips.hpp:609-636 for nv = 3): removing c0 leaves
// (c1, c2), removing c1 leaves (c0, c2), removing c2 leaves (c0, c1).
template <typename Cx>
__device__ __forceinline__ u64 tri_zero_facet(const Cx& cx, u32 c0, u32 c1, u32 c2, f32 d, u32& f0, u32& f1) {
    if (cx.d(c1, c2) == d) { f0 = c1; f1 = c2; return edge_idx(c1, c2); }
    if (cx.d(c0, c2) == d) { f0 = c0; f1 = c2; return edge_idx(c0, c2); }
    if (cx.d(c0, c1) == d) { f0 = c0; f1 = c1; return edge_idx(c0, c1); }
    return kNone;
}

// Rows of the complex as edge sources: row v lists its neighbours u < v in
// increasing u (the dense matrix's row prefix, or the sorted CSR row).
struct DenseRows {
    const f32* mat;
    u32 n;
    __device__ __forceinline__ u64 begin(u32) const { return 0; }
    __device__ __forceinline__ u64 end(u32 v) const { return v; }
    __device__ __forceinline__ void at(u32 v, u64 t, u32& u, f32& d) const {
        u = u32(t);
        d = mat[u64(v) * n + t];
    }
};
struct CsrRows {
    const u64* rp;
    const u32* ci;
    const f32* w;
    __device__ __forceinline__ u64 begin(u32 v) const { return rp[v]; }
    __device__ __forceinline__ u64 end(u32 v) const { return rp[v + 1]; }
    __device__ __forceinline__ void at(u32, u64 t, u32& u, f32& d) const {
        u = ci[t];
        d = w[t];
    }
};

// cnt[v] = kept edges {u, v}: u < v, d(u, v) <= thr (one warp per row);
// dmm[0] / dmm[1] = the smallest / largest distance bits kept (the sort's
// bit range, known with the count).
template <typename Rows>
__global__ void k_edge_count(Rows rows, u32 n, f32 thr, u64* __restrict__ cnt, u32* __restrict__ dmm) {
    pdl_wait();
    pdl_trigger();
    const int lane = threadIdx.x & 31;
    const u32 warps = (gridDim.x * blockDim.x) >> 5;
    u32 lo = 0xffffffffu, hi = 0;
    for (u32 v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += warps) {
        const u64 b = rows.begin(v), e = rows.end(v);
        u32 c = 0;
        for (u64 t0 = b; t0 < e; t0 += 32) {
            bool keep = false;
            if (t0 + lane < e) {
                u32 u;
                f32 d;
                rows.at(v, t0 + lane, u, d);
                keep = u < v && d <= thr;
                if (keep) {
                    lo = min(lo, __float_as_uint(d));
                    hi = max(hi, __float_as_uint(d));
                }
            }
            c += __popc(__ballot_sync(0xffffffffu, keep));
        }
        if (lane == 0) cnt[v] = c;
    }
    // one atomic pair per block
    __shared__ u32 blo, bhi;
    if (threadIdx.x == 0) {
        blo = 0xffffffffu;
        bhi = 0;
    }
    __syncthreads();
    lo = __reduce_min_sync(0xffffffffu, lo);
    hi = __reduce_max_sync(0xffffffffu, hi);
    if (lane == 0 && lo <= hi) {
        atomicMin(&blo, lo);
        atomicMax(&bhi, hi);
    }
    __syncthreads();
    if (threadIdx.x == 0 && blo <= bhi) {
        atomicMin(&dmm[0], blo);
        atomicMax(&dmm[1], bhi);
    }
}

// Kept edges in a fixed order: position p = off[v] + rank in row runs over
// edge indices in increasing order (rows ascending, u ascending within a
// row). Entry q (q = m - 1 - p for the Ripser order, idx descending; q = p
// for the RedZeD order, idx ascending) gets sort key dbits << 32 | q and
// idx. A stable sort on the dbits then yields (d, idx) in the filtration
// order: the ties keep the order of q.
template <typename Rows>
__global__ void k_edge_fill(Rows rows, u32 n, f32 thr, const u64* __restrict__ off, u64 m, int redzed,
                            u64* __restrict__ skey, u64* __restrict__ sidx, u32* __restrict__ err) {
    pdl_wait();
    pdl_trigger();
    const int lane = threadIdx.x & 31;
    const u32 warps = (gridDim.x * blockDim.x) >> 5;
    for (u32 v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += warps) {
        const u64 b = rows.begin(v), e = rows.end(v);
        const u64 vbase = u64(v) * (v - 1) / 2;
        u64 base = off[v];
        for (u64 t0 = b; t0 < e; t0 += 32) {
            bool keep = false;
            u32 u = 0;
            f32 d = 0.0f;
            if (t0 + lane < e) {
                rows.at(v, t0 + lane, u, d);
                keep = u < v && d <= thr;
            }
            const u32 bal = __ballot_sync(0xffffffffu, keep);
            if (keep) {
                const u64 p = base + __popc(bal & ((1u << lane) - 1));
                if (p < m) {
                    const u64 q = redzed ? p : m - 1 - p;
                    skey[q] = (u64(__float_as_uint(d)) << 32) | q;
                    sidx[q] = vbase + u;
                } else if (err) {
                    atomicOr(err, 1u);   // more kept edges than the caller announced
                }
            }
            base += __popc(bal);
        }
    }
}

// Sorted (dbits, q) pairs -> filtration keys (packed, or as they are in the
// wide layout, where sidx stays the index table); inv[q] = sorted position of
// the edge that index order puts at q.
__global__ void k_edge_pack(const u64* __restrict__ skey, const u64* __restrict__ sidx, u64 m, int redzed, int wide,
                            u64* __restrict__ keys, u32* __restrict__ inv) {
    pdl_wait();
    pdl_trigger();
    for (u64 r = u64(blockIdx.x) * blockDim.x + threadIdx.x; r < m; r += u64(gridDim.x) * blockDim.x) {
        const u64 k = skey[r];
        if (wide) {
            keys[r] = k;
        } else {
            const u64 idx = sidx[u32(k)];
            keys[r] = ((k >> 32) << kIdxBits) | (redzed ? idx : kIdxMask - idx);
        }
        inv[u32(k)] = u32(r);
    }
}

__global__ void k_apparent_dense(const f32* __restrict__ mat, u32 n, const u64* __restrict__ keys, EdgeFmt fmt, u64 m,
                                 u8* __restrict__ app, u32* __restrict__ emw, u8* __restrict__ emf) {
    pdl_wait();
    pdl_trigger();
    const DenseCx cx{mat, n};
    const int lane = threadIdx.x & 31;
    const u64 warps = (u64(gridDim.x) * blockDim.x) >> 5;
    for (u64 e = (u64(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; e < m; e += warps) {
        const u64 key = keys[e];
        const f32 d = fmt.d(key);
        const u64 idx = fmt.rips(key);
        u32 a, b;
        decode_edge(idx, a, b);
        const u32 w = warp_top_cofacet2(cx, a, b, d);
        bool apparent = false, em = false;
        if (w != NOV) {
            u32 c0 = a, c1 = b, c2 = w;
            sort3(c0, c1, c2);
            u32 f0 = 0, f1 = 0;
            const u64 f = tri_zero_facet(cx, c0, c1, c2, d, f0, f1);
            apparent = f == idx;
            if (!apparent) {
                // emergent probe: does the cofacet have a zero-apparent facet?
                // Its zero facet is (f0, f1); that facet's zero cofacet must
                // be the same triangle.
                const u32 w2 = warp_top_cofacet2(cx, f0, f1, d);
                if (w2 != NOV) {
                    u32 g0 = f0, g1 = f1, g2 = w2;
                    sort3(g0, g1, g2);
                    em = g0 == c0 && g1 == c1 && g2 == c2;
                }
            }
        }
        if (lane == 0) {
            app[e] = apparent;
            emw[e] = w;
            emf[e] = em;
        }
    }
}

// --------------------------------------------------------------------------
// Sparse complex (CSR, rows ascending).
// --------------------------------------------------------------------------
struct CsrCx {
    const u64* rp;
    const u32* ci;
    const f32* w;
    // Largest common neighbour x of a and b with both weights <= cap (the
    // k-way intersection walked from the top, rips.hpp:429-471), and its two
    // weights w(a, x), w(b, x).
    __device__ __forceinline__ u32 top_cofacet2(u32 a, u32 b, f32 cap, f32& wax, f32& wbx) const {
        u64 pa = rp[a + 1], pb = rp[b + 1];
        const u64 la = rp[a], lb = rp[b];
        while (pa > la && pb > lb) {
            const u32 xa = ci[pa - 1], xb = ci[pb - 1];
            if (xa > xb) { --pa; continue; }
            if (xb > xa) { --pb; continue; }
            const f32 x1 = w[pa - 1], x2 = w[pb - 1];
            if (x1 <= cap && x2 <= cap) {
                wax = x1;
                wbx = x2;
                return xa;
            }
            --pa;
            --pb;
        }
        return NOV;
    }
};

// Edges are visited in index order (inv: index order -> sorted position), so
// neighbouring threads share the larger vertex's row; results go to the
// edge's sorted position.
// (32 registers: 64 warps an SM to hide the walk's load latency.)
__global__ void __launch_bounds__(256, 8)
    k_apparent_csr(CsrCx cx, const u64* __restrict__ keys, EdgeFmt fmt, const u32* __restrict__ inv, u64 m,
                   u8* __restrict__ app, u32* __restrict__ emw, u8* __restrict__ emf) {
    pdl_wait();
    pdl_trigger();
    for (u64 t = u64(blockIdx.x) * blockDim.x + threadIdx.x; t < m; t += u64(gridDim.x) * blockDim.x) {
        const u64 e = inv[t];
        const u64 key = keys[e];
        const f32 d = fmt.d(key);
        const u64 idx = fmt.rips(key);
        u32 a, b;
        decode_edge(idx, a, b);
        f32 wax = 0.0f, wbx = 0.0f;
        const u32 w = cx.top_cofacet2(a, b, d, wax, wbx);
        bool apparent = false, em = false;
        if (w != NOV) {
            u32 c0 = a, c1 = b, c2 = w;
            sort3(c0, c1, c2);
            // the zero facet (tri_zero_facet's order) from the three known
            // edge lengths: (a, b) = d, (a, w) = wax, (b, w) = wbx
            auto len = [&](u32 u, u32 v) -> f32 {
                if ((u == a && v == b) || (u == b && v == a)) return d;
                return u == a || v == a ? wax : wbx;
            };
            u32 f0, f1;
            if (len(c1, c2) == d) f0 = c1, f1 = c2;
            else if (len(c0, c2) == d) f0 = c0, f1 = c2;
            else f0 = c0, f1 = c1;   // (a, b) is one of the three pairs: one length equals d
            apparent = edge_idx(f0, f1) == idx;
            if (!apparent) {
                f32 t1, t2;
                const u32 w2 = cx.top_cofacet2(f0, f1, d, t1, t2);
                if (w2 != NOV) {
                    u32 g0 = f0, g1 = f1, g2 = w2;
                    sort3(g0, g1, g2);
                    em = g0 == c0 && g1 == c1 && g2 == c2;
                }
            }
        }
        app[e] = apparent;
        emw[e] = w;
        emf[e] = em;
    }
}

// --------------------------------------------------------------------------
// Borůvka over edge ranks (rank = position in the sorted array).
// --------------------------------------------------------------------------
__global__ void k_iota(u32* __restrict__ p, u32 n) {
    pdl_wait();
    pdl_trigger();
    for (u32 v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) p[v] = v;
}

// For each live edge with endpoints in different components, offer its rank
// to both components; edges inside a component are dropped from the list.
// (The survivors' list grows by one atomic per warp: ranks from a ballot.
// The first round offers all m edges; later rounds read their count from
// the previous round's counter, so rounds run without a host round trip.)
__global__ void k_bv_offer(const u64* __restrict__ keys, EdgeFmt fmt, const u32* __restrict__ live,
                           const u32* __restrict__ nlive_in, u32 m, const u32* __restrict__ comp,
                           u32* __restrict__ best, u32* __restrict__ live_out, u32* __restrict__ nlive_out) {
    pdl_wait();
    pdl_trigger();
    const u32 lane = threadIdx.x & 31;
    const bool all = nlive_in == nullptr;
    const u32 nlive = all ? m : *nlive_in;
    for (u32 base = blockIdx.x * blockDim.x; base < nlive; base += gridDim.x * blockDim.x) {
        const u32 t = base + threadIdx.x;   // whole warps iterate together
        bool keep = false;
        u32 r = 0;
        if (t < nlive) {
            r = all ? t : live[t];
            u32 a, b;
            decode_edge(fmt.rips(keys[r]), a, b);
            const u32 ca = comp[a], cb = comp[b];
            if (ca != cb) {
                atomicMin(&best[ca], r);
                atomicMin(&best[cb], r);
                keep = true;
            }
        }
        const u32 m = __ballot_sync(0xffffffffu, keep);
        if (!m) continue;
        u32 pos = 0;
        if (lane == u32(__ffs(m) - 1)) pos = atomicAdd(nlive_out, u32(__popc(m)));
        pos = __shfl_sync(0xffffffffu, pos, __ffs(m) - 1);
        if (keep) live_out[pos + __popc(m & ((1u << lane) - 1u))] = r;
    }
}

// Every component root with an offered edge takes it into the forest and
// hooks onto the other side; of a mutual pair only the larger root hooks.
// (The hook count is summed per warp: one atomic a warp. A round whose offer
// found no edge between components has nothing to hook: live == 0.)
__global__ void k_bv_hook(const u64* __restrict__ keys, EdgeFmt fmt, const u32* __restrict__ comp,
                          const u32* __restrict__ best,
                          u32* __restrict__ parent, u8* __restrict__ tree, u32 n, u32* __restrict__ hooks,
                          const u32* __restrict__ live) {
    pdl_wait();
    pdl_trigger();
    if (*live == 0) return;
    u32 mine = 0;
    for (u32 c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        if (comp[c] != c) continue;
        const u32 r = best[c];
        if (r == NOV) continue;
        u32 a, b;
        decode_edge(fmt.rips(keys[r]), a, b);
        const u32 o = comp[a] == c ? comp[b] : comp[a];
        tree[r] = 1;
        if (best[o] == r && c < o) continue;   // mutual: o hooks onto c
        parent[c] = o;
        ++mine;
    }
    mine = __reduce_add_sync(0xffffffffu, mine);
    if ((threadIdx.x & 31) == 0 && mine) atomicAdd(hooks, mine);
}

__global__ void k_bv_flatten(const u32* __restrict__ parent, u32* __restrict__ comp, u32* __restrict__ best, u32 n,
                             const u32* __restrict__ live) {
    pdl_wait();
    pdl_trigger();
    if (*live == 0) return;   // no hook this round: parents, components and offers unchanged
    for (u32 v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        u32 r = parent[v];
        for (u32 s = 0; parent[r] != r && s < n; ++s) r = parent[r];
        comp[v] = r;
        best[v] = NOV;
    }
}

// --------------------------------------------------------------------------
// Ordered compaction of H0 bars and columns.
// --------------------------------------------------------------------------
// One flag word per edge: finite H0 bar << 32 | column (m < 2^32, so one
// scan counts both without a carry between the halves).
__global__ void k_flags_dim0(const u64* __restrict__ keys, EdgeFmt fmt, const u8* __restrict__ tree,
                             const u8* __restrict__ app, u64 m, int want_cols, u64* __restrict__ f) {
    pdl_wait();
    pdl_trigger();
    for (u64 e = u64(blockIdx.x) * blockDim.x + threadIdx.x; e < m; e += u64(gridDim.x) * blockDim.x) {
        const bool t = tree[e];
        f[e] = (u64(t && fmt.d(keys[e]) > 0.0f) << 32) | u64(want_cols && !t && !(app && app[e]));
    }
}

__global__ void k_emit_dim0(const u64* __restrict__ keys, EdgeFmt fmt, const u8* __restrict__ tree,
                            const u8* __restrict__ app,
                            const u32* __restrict__ emw, const u8* __restrict__ emf, u64 m, int want_cols,
                            const u64* __restrict__ o2, const u64* __restrict__ tot,
                            f32* __restrict__ h0, u64* __restrict__ h0_edge, u64* __restrict__ cidx,
                            f32* __restrict__ cd, u64* __restrict__ emi, u8* __restrict__ emf_out) {
    pdl_wait();
    pdl_trigger();
    const u64 ncols = tot[0] & 0xffffffffull;
    for (u64 e = u64(blockIdx.x) * blockDim.x + threadIdx.x; e < m; e += u64(gridDim.x) * blockDim.x) {
        const u64 key = keys[e];
        const f32 d = fmt.d(key);
        const bool t = tree[e];
        const u64 oe = o2[e];   // exclusive counts: H0 bars << 32 | columns
        if (t && d > 0.0f) {
            h0[oe >> 32] = d;
            h0_edge[oe >> 32] = fmt.rips(key);   // the bar's critical (death) edge
        }
        if (want_cols && !t && !(app && app[e])) {
            const u64 o = ncols - 1 - (oe & 0xffffffffull);   // descending order (rips.hpp:867)
            const u64 idx = fmt.rips(key);
            cidx[o] = idx;
            cd[o] = d;
            const u32 w = emw[e];
            if (w == NOV) {
                emi[o] = kNone;
                emf_out[o] = 0;
            } else {
                u32 a, b;
                decode_edge(idx, a, b);
                u32 c0 = a, c1 = b, c2 = w;
                sort3(c0, c1, c2);
                emi[o] = tri_idx(c0, c1, c2);
                emf_out[o] = emf[e];
            }
        }
    }
}


inline u32 grid_for(u64 work, u32 per_block) {
    const u64 g = (work + per_block - 1) / per_block;
    return u32(std::max<u64>(1, std::min<u64>(g, 64ull * kSMs)));
}

}  // namespace

// Kept edges as sorted keys (Ripser or RedZeD order); returns the count.
// The edges are written in index order (count, scan, fill), so one stable
// sort on the distance bits alone gives the filtration order: only the bits
// in which the kept distances differ (their range comes back with the count),
// three passes when 25 bits differ, instead of a full 64-bit key sort.
// Slots: S_EDGE_CNT, S_EDGE_SORT, S_EDGE_IDX, S_EDGE_KEYS (result),
// S_EDGE_INV (result: index order -> sorted position),
// and the sort's own (S_SORT_A, S_SORT_HIST, S_SCAN*, S_MISC3).
// Above kPackedMaxN vertices the keys take the wide layout (EdgeFmt) and
// *eidx_out the index table; otherwise *eidx_out is null. m_known (not
// kUnknownM): the caller knows the kept-edge count (a symmetric graph without
// self loops cut at +inf keeps nnz / 2), so the count is not read back: the
// sort takes all 31 distance bits, and a wrong count sets *err instead of
// writing out of bounds.
constexpr u64 kUnknownM = ~0ull;
static u64 sorted_edge_keys(tt_ctx* c, const Complex& cx, int redzed, u64** keys_out, u64** eidx_out,
                            u64 m_known = kUnknownM, u32* err = nullptr) {
    const u32 n = cx.n;
    u64 m = 0;
    u64* off = c->arena.get<u64>(S_EDGE_CNT, u64(n) + 2);
    u32* dmm = reinterpret_cast<u32*>(off + n + 1);   // beside the total: one copy brings both
    const u32 g = grid_for(u64(n) * 32, 256);
    int dbits = 0;   // distance bits the sort must see
    if (n > 1) {
        TT_CUDA(cudaMemsetAsync(dmm, 0xff, sizeof(u32), c->stream));
        TT_CUDA(cudaMemsetAsync(dmm + 1, 0, sizeof(u32), c->stream));
        if (cx.mat)
            launch_pdl(k_edge_count<DenseRows>, g, 256, 0, c->stream, DenseRows{cx.mat, n}, n, cx.thr, off, dmm);
        else
            launch_pdl(k_edge_count<CsrRows>, g, 256, 0, c->stream, CsrRows{cx.rp, cx.ci, cx.w}, n, cx.thr, off, dmm);
        TT_LAUNCH("k_edge_count");
        ++c->launches;
        scan_exclusive<u64>(c, off, off, n, off + n);
        if (m_known != kUnknownM) {
            m = m_known;
            dbits = 31;   // every bit of a non-negative float: the same three passes
        } else {
            u64 h[2];
            TT_CUDA(cudaMemcpyAsync(h, off + n, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
            TT_CUDA(cudaStreamSynchronize(c->stream));
            m = h[0];
            const u32 lo = u32(h[1]), hi = u32(h[1] >> 32);
            const u32 diff = m ? lo ^ hi : 0u;
            dbits = diff ? 32 - __builtin_clz(diff) : 0;
        }
    }
    if (m >= 0xffffffffull) invalid("gb300: more than 2^32 - 1 kept edges");
    u64* keys = c->arena.get<u64>(S_EDGE_KEYS, m + 1);
    const bool wide = n > kPackedMaxN;
    *eidx_out = nullptr;
    if (m) {
        u64* skey = c->arena.get<u64>(S_EDGE_SORT, m + 1);
        u64* sidx = c->arena.get<u64>(S_EDGE_IDX, m + 1);
        if (cx.mat)
            launch_pdl(k_edge_fill<DenseRows>, g, 256, 0, c->stream, DenseRows{cx.mat, n}, n, cx.thr, off, m, redzed, skey,
                       sidx, err);
        else
            launch_pdl(k_edge_fill<CsrRows>, g, 256, 0, c->stream, CsrRows{cx.rp, cx.ci, cx.w}, n, cx.thr, off, m, redzed,
                       skey, sidx, err);
        TT_LAUNCH("k_edge_fill");
        u64* kb = c->arena.get<u64>(S_SORT_A, m);
        // a stable sort on the distance bits that differ (none: already in order)
        const bool sw = dbits > 0 && radix_sort<u32>(c, skey, static_cast<u32*>(nullptr), m, kb,
                                                     static_cast<u32*>(nullptr), dbits, 32);
        u32* inv = c->arena.get<u32>(S_EDGE_INV, m + 1);
        launch_pdl(k_edge_pack, grid_for(m, 256), 256, 0, c->stream, sw ? kb : skey, sidx, m, redzed, wide, keys, inv);
        if (wide) *eidx_out = sidx;
        TT_LAUNCH("k_edge_pack");
        c->launches += 2;
    }
    *keys_out = keys;
    return m;
}

void dim0(tt_ctx* c, const Complex& cx, u32 maxdim, Dim0Out& out, u64 m_known) {
    out = Dim0Out{};
    u32* err = m_known != kUnknownM ? c->arena.get<u32>(S_DIM0_ERR, 4) : nullptr;
    if (err) TT_CUDA(cudaMemsetAsync(err, 0, sizeof(u32), c->stream));
    const u64 m = sorted_edge_keys(c, cx, 0, &out.keys, &out.eidx, m_known, err);
    const EdgeFmt fmt{out.eidx};
    out.m = m;
    if (m >= 0xffffffffull) invalid("gb300: more than 2^32 - 1 kept edges");
    const u32 n = cx.n;
    // per-edge flags
    u8* app = c->arena.get<u8>(S_FLAGS, 2 * m + 16);
    u8* tree = app + m + 8;
    u32* emw = c->arena.get<u32>(S_EDGE_TMP, m + 1);
    u8* emf = c->arena.get<u8>(S_MISC2, m + 1);
    TT_CUDA(cudaMemsetAsync(tree, 0, m + 1, c->stream));
    // The apparent/emergent scan and the spanning forest read the same sorted
    // edges and write disjoint flags. The forest's short rounds (and their
    // host round trips) run on the side stream, which has the highest
    // priority: its blocks are scheduled ahead of the scan's waiting blocks,
    // and the scan, on the main stream, fills the SMs around them.
    SideScope side(c);
    const cudaStream_t fs = n ? side.fork() : c->stream;   // the forest's stream
    if (maxdim >= 1 && m) {
        u32* inv = c->arena.get<u32>(S_EDGE_INV, m + 1);
        const cudaStream_t s = c->stream;
        if (cx.mat)
            launch_pdl(k_apparent_dense, grid_for(m * 32, 256), 256, 0, s, cx.mat, n, out.keys, fmt, m, app, emw, emf);
        else
            // six of the eight resident blocks an SM: the forest's short
            // kernels then always find free slots instead of waiting for a
            // wave of scan blocks to retire (measured: kNN front end of
            // 100,000 points, dim0 0.04 ms shorter than with all eight)
            launch_pdl(k_apparent_csr, std::min<u32>(grid_for(m, 256), 6 * kSMs), 256, 0, s, 
                CsrCx{cx.rp, cx.ci, cx.w}, out.keys, fmt, inv, m, app, emw, emf);
        TT_LAUNCH("k_apparent");
        ++c->launches;
    }
    out.app = maxdim >= 1 ? app : nullptr;
    out.tree = tree;
    // Borůvka spanning forest
    u32* comp = c->arena.get<u32>(S_UF_PARENT, 2 * u64(n) + 2);
    u32* parent = comp + n + 1;
    u32* best = c->arena.get<u32>(S_UF_BEST, n + 1);
    u32* live0 = c->arena.get<u32>(S_UF_WORK, m + 1);
    u32* live1 = c->arena.get<u32>(S_UF_WORK2, m + 1);
    constexpr int kRounds = 64, kPerTrip = 3;
    u32* ctr = c->arena.get<u32>(S_MISC1, 2 * kRounds);   // per round: live count, hooks
    u64 total_hooks = 0;
    if (n) {
        launch_pdl(k_iota, grid_for(n, 256), 256, 0, fs, comp, n);
        launch_pdl(k_iota, grid_for(n, 256), 256, 0, fs, parent, n);
        TT_CUDA(cudaMemsetAsync(best, 0xff, sizeof(u32) * n, fs));
        c->launches += 2;
        TT_CUDA(cudaMemsetAsync(ctr, 0, 2 * kRounds * sizeof(u32), fs));
        // Three rounds a host round trip (a round after convergence finds no
        // edge between components and changes nothing); the grid covers the
        // last live count the host knows (counts only shrink).
        u32 known = u32(m);
        for (int round = 0; known && round < kRounds;) {
            const int first = round;
            for (int q = 0; q < kPerTrip && round < kRounds; ++q, ++round) {
                launch_pdl(k_bv_offer, grid_for(known, 256), 256, 0, fs, 
                    out.keys, fmt, live0, round ? ctr + 2 * (round - 1) : nullptr, u32(m), comp, best, live1, ctr + 2 * round);
                launch_pdl(k_bv_hook, grid_for(n, 256), 256, 0, fs, out.keys, fmt, comp, best, parent, tree, n,
                                                           ctr + 2 * round + 1, ctr + 2 * round);
                launch_pdl(k_bv_flatten, grid_for(n, 256), 256, 0, fs, parent, comp, best, n, ctr + 2 * round);
                TT_LAUNCH("boruvka");
                c->launches += 3;
                std::swap(live0, live1);
            }
            u32 h[2 * kPerTrip] = {};
            TT_CUDA(cudaMemcpyAsync(h, ctr + 2 * first, sizeof(u32) * 2 * (round - first), cudaMemcpyDeviceToHost,
                                    fs));
            TT_CUDA(cudaStreamSynchronize(fs));
            const int last = round - first - 1;
            for (int q = 0; q <= last; ++q) total_hooks += h[2 * q + 1];
            known = h[2 * last];
            if (h[2 * last + 1] == 0) break;
        }
    }
    side.join();   // the forest's tree flags
    // ordered compaction of H0 deaths and columns
    const int want_cols = maxdim >= 1;
    u64* f2 = c->arena.get<u64>(S_MISC0, 2 * m + 4);
    u64* o2 = f2 + m + 2;
    u64* tot = c->arena.get<u64>(S_COUNT, 4);
    if (m) {
        launch_pdl(k_flags_dim0, grid_for(m, 256), 256, 0, c->stream, out.keys, fmt, tree, out.app, m, want_cols, f2);
        TT_LAUNCH("k_flags_dim0");
        scan_exclusive<u64>(c, f2, o2, m, tot);
        c->launches += 1;
    } else {
        TT_CUDA(cudaMemsetAsync(tot, 0, sizeof(u64), c->stream));
    }
    // the outputs: at their largest sizes (H0 bars < n, columns <= m) when
    // that is small, so the emit is enqueued before the counts come back;
    // otherwise at the counted sizes, after the round trip
    auto emit = [&](u64 nh0, u64 ncols) {
        out.h0 = c->arena.get<f32>(S_OUT0, nh0 + 1);
        out.cidx = c->arena.get<u64>(S_OUT1, ncols + 1);
        out.cd = c->arena.get<f32>(S_OUT2, ncols + 1);
        out.emi = c->arena.get<u64>(S_OUT3, ncols + 1);
        out.emf = c->arena.get<u8>(S_OUT4, ncols + 1);
        out.h0_edge = c->arena.get<u64>(S_OUT5, nh0 + 1);
        if (m) {
            launch_pdl(k_emit_dim0, grid_for(m, 256), 256, 0, c->stream, out.keys, fmt, tree, out.app, emw, emf, m, want_cols,
                                                                 o2, tot, out.h0, out.h0_edge, out.cidx, out.cd,
                                                                 out.emi, out.emf);
            TT_LAUNCH("k_emit_dim0");
            ++c->launches;
        }
    };
    const bool early = m <= (u64(1) << 24);
    if (early) emit(n, want_cols ? m : 0);
    u64 hp = 0;
    u32 bad = 0;
    TT_CUDA(cudaMemcpyAsync(&hp, tot, sizeof(hp), cudaMemcpyDeviceToHost, c->stream));
    if (err) TT_CUDA(cudaMemcpyAsync(&bad, err, sizeof(bad), cudaMemcpyDeviceToHost, c->stream));
    TT_CUDA(cudaStreamSynchronize(c->stream));
    if (bad) throw Error(TT_ERR_INTERNAL, "gb300: more kept edges than announced");
    const u64 h[2] = {hp >> 32, hp & 0xffffffffull};
    out.nh0 = h[0];
    out.ncols = h[1];
    if (!early) emit(h[0], h[1]);
    // every hook merged two components through one tree edge
    out.essential = n - total_hooks;
}

namespace {
__global__ void k_emit_redzed(const u64* __restrict__ keys, EdgeFmt fmt, u64 m, f32* __restrict__ d,
                              int32_t* __restrict__ v) {
    for (u64 e = u64(blockIdx.x) * blockDim.x + threadIdx.x; e < m; e += u64(gridDim.x) * blockDim.x) {
        const u64 k = keys[e];
        u32 a, b;
        decode_edge(fmt.redzed(k), a, b);
        d[e] = fmt.d(k);
        v[2 * e] = int32_t(b);
        v[2 * e + 1] = int32_t(a);
    }
}
}  // namespace

// redzed::detail::build_edges (redzed.hpp:545-613): kept edges in
// (d asc, combinatorial index asc) order, vertices (i < j). Writes up to cap
// edges to the device buffers d / verts and returns the edge count.
u64 redzed_edges(tt_ctx* c, const Complex& cx, f32* d, int32_t* verts, u64 cap) {
    u64* keys = nullptr;
    u64* eidx = nullptr;
    const u64 m = sorted_edge_keys(c, cx, 1, &keys, &eidx);
    if (m && m <= cap) {
        k_emit_redzed<<<grid_for(m, 256), 256, 0, c->stream>>>(keys, EdgeFmt{eidx}, m, d, verts);
        TT_LAUNCH("k_emit_redzed");
        ++c->launches;
    }
    return m;
}

// The same edge list in context-owned device arrays sized to its count
// (slots S_RZ_D / S_RZ_V), for the host-buffer entry points.
u64 redzed_edges_owned(tt_ctx* c, const Complex& cx, f32** d, int32_t** verts) {
    u64* keys = nullptr;
    u64* eidx = nullptr;
    const u64 m = sorted_edge_keys(c, cx, 1, &keys, &eidx);
    *d = c->arena.get<f32>(S_RZ_D, m + 1);
    *verts = c->arena.get<int32_t>(S_RZ_V, 2 * m + 2);
    if (m) {
        k_emit_redzed<<<grid_for(m, 256), 256, 0, c->stream>>>(keys, EdgeFmt{eidx}, m, *d, *verts);
        TT_LAUNCH("k_emit_redzed");
        ++c->launches;
    }
    return m;
}

}  // namespace tt
