// tt_internal.cuh — declarations shared by the library's translation units.
#pragma once
#include "tt_common.cuh"

namespace tt {

// Packed filtration keys for edges and triangles: the float bits of the
// diameter (non-negative, so integer order == float order; < 2^31) above a
// 33-bit simplex index. Ripser order (rips.hpp:114-118) is (d asc, idx desc):
// the index field holds kIdxMask - idx. RedZeD order (redzed.hpp:477-480) is
// (d asc, combinatorial index asc): the field holds idx. Indices must be
// < 2^33 (edges: n <= 131072; triangles: C(n, 3) < 2^33).
constexpr int kIdxBits = 33;
constexpr u64 kIdxMask = (1ull << kIdxBits) - 1;
__host__ __device__ inline u64 key_rips(f32 d, u64 idx) {
    return (u64(fbits(d)) << kIdxBits) | (kIdxMask - idx);
}

// Edge indices fit the packed key's 33-bit field while n <= kPackedMaxN.
constexpr u32 kPackedMaxN = 131072;

// Simplex index helpers (combinatorial number system, rips.hpp:505-580).
// Programmatic dependent launch: a kernel launched with launch_pdl may start
// while the previous kernel of its stream finishes; pdl_wait (first thing in
// such a kernel) waits until that kernel has completed and its writes are
// visible, and pdl_trigger lets the next one start. Both do nothing in a
// kernel launched the ordinary way.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
void launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    TT_CUDA(cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...));
}

__device__ __forceinline__ void decode_edge(u64 idx, u32& a, u32& b) {
    // rips.hpp decode, nv = 2 closed form (:549-557): a > b. The FP32 closed
    // form is within one of the answer for idx < 2^40 (relative error below
    // 2^-23 on a root below 2^21), the FP64 one for every 64-bit idx; the
    // integer steps make it exact.
    u64 v = idx < (1ull << 40) ? u64((1.0f + sqrtf(fmaf(8.0f, float(idx), 1.0f))) * 0.5f)
                               : u64((1.0 + sqrt(fma(8.0, double(idx), 1.0))) * 0.5);
    while (v * (v - 1) / 2 > idx) --v;
    while ((v + 1) * v / 2 <= idx) ++v;
    a = u32(v);
    b = u32(idx - v * (v - 1) / 2);
}
__device__ __forceinline__ u64 edge_idx(u32 a, u32 b) {   // any order
    if (a < b) { const u32 t = a; a = b; b = t; }
    return u64(a) * (a - 1) / 2 + b;
}
__device__ __forceinline__ u64 tri_idx(u32 a, u32 b, u32 c) {   // a > b > c
    return u64(a) * (a - 1) * (a - 2) / 6 + u64(b) * (b - 1) / 2 + c;
}
__device__ __forceinline__ void sort3(u32& a, u32& b, u32& c) {   // descending
    if (a < b) { const u32 t = a; a = b; b = t; }
    if (b < c) { const u32 t = b; b = c; c = t; }
    if (a < b) { const u32 t = a; a = b; b = t; }
}
__device__ __forceinline__ f32 key_d(u64 k) { return __uint_as_float(u32(k >> kIdxBits)); }
__device__ __forceinline__ u64 key_idx(u64 k) { return kIdxMask - (k & kIdxMask); }

// Sorted edge keys come in two layouts. Packed (eidx == nullptr, n <=
// kPackedMaxN): float bits of d << 33 | the index field above. Wide (larger
// n, whose edge indices need more than 33 bits): float bits of d << 32 | q,
// q the edge's position among the kept edges in index order (descending for
// the Ripser order, ascending for RedZeD's, so that integer order is still
// the filtration order), and eidx[q] the edge's index.
struct EdgeFmt {
    const u64* eidx = nullptr;
    __device__ __forceinline__ f32 d(u64 k) const { return eidx ? __uint_as_float(u32(k >> 32)) : key_d(k); }
    __device__ __forceinline__ u64 rips(u64 k) const { return eidx ? eidx[u32(k)] : key_idx(k); }
    __device__ __forceinline__ u64 redzed(u64 k) const { return eidx ? eidx[u32(k)] : (k & kIdxMask); }
};


// ---- tt_dense.cu
void dense_matrix(tt_ctx* c, const f32* x, u32 n, u32 dim, int kind, f32 p, f32* mat, u32* rowmax);
void min_bits(tt_ctx* c, const u32* v, u32 n, u32* out);

// ---- tt_sort.cu
template <typename T>
void scan_exclusive(tt_ctx* c, const T* in, T* out, u64 n, T* total, int depth = 0);
// Stable LSD sort on key bits [lo_bit, 64); the bits above lo_bit are sorted
// as far as the keys differ there (force_bits > 0: exactly that many).
template <typename V>
bool radix_sort(tt_ctx* c, u64* keys, V* vals, u64 n, u64* kbuf, V* vbuf, int force_bits = 0, int lo_bit = 0,
                const unsigned long long* ndev = nullptr);
template <typename V>
void radix_sort_inplace(tt_ctx* c, u64* keys, V* vals, u64 n, int force_bits = 0);
void radix_reserve(tt_ctx* c, u64 n);   // every slot radix_sort of n keys may grow
void radix_reserve_entries(tt_ctx* c, u64 entries);   // ... a sort whose histogram has that many entries
// A tile of the segmented sort: tile t (of tcount) of segment seg; its digit
// counts at hbase + digit * tcount + t (segments' count blocks in segment
// order, each 256 * tcount entries).
struct SegTile {
    u32 seg, t, hbase, tcount;
};
constexpr u32 kSegTileKeys = 4096;   // keys a tile of the segmented sort
bool radix_sort_segments(tt_ctx* c, u64* keys, u64* kbuf, const u64* seg_off, const SegTile* tl,
                         const u32* ntiles_dev, u32 max_tiles, u64 hist_entries, int bits, int lo_bit);

// ---- tt_dim0.cu
struct Dim0Out {
    u64 m = 0;            // kept edges
    u64* keys = nullptr;  // m sorted Ripser keys (device)
    u64* eidx = nullptr;  // wide layout (n > kPackedMaxN): edge index by index-order position
    u8* app = nullptr;    // m apparent flags (device), maxdim >= 1
    u8* tree = nullptr;   // m spanning-tree flags (device)
    u64 ncols = 0;        // dim-1 columns
    u64* cidx = nullptr;  // columns (device), descending filtration order
    f32* cd = nullptr;
    u64* emi = nullptr;   // emergent probe per column: first zero cofacet index or kNone
    u8* emf = nullptr;    //   and whether that cofacet has a zero-apparent facet
    u64 nh0 = 0;          // finite H0 bars (d > 0), sorted edge order
    f32* h0 = nullptr;    // deaths (device)
    u64* h0_edge = nullptr;   // each finite H0 bar's tree edge (edge index, device)
    u64 essential = 0;    // connected components
};
// Graph is either a dense full matrix (mat != nullptr) or a CSR.
struct Complex {
    const f32* mat = nullptr;
    const u64* rp = nullptr;
    const u32* ci = nullptr;
    const f32* w = nullptr;
    u32 n = 0;
    f32 thr = 0;
};
// m_known: the kept-edge count when the caller knows it (a symmetric graph
// without self loops cut at +inf keeps nnz / 2); saves the round trip that
// would read it back.
void dim0(tt_ctx* c, const Complex& cx, u32 maxdim, Dim0Out& out, u64 m_known = ~0ull);
// RedZeD EdgeList (d asc, comb asc): diam + vertex pairs (i < j).
u64 redzed_edges(tt_ctx* c, const Complex& cx, f32* d, int32_t* verts, u64 cap);
u64 redzed_edges_owned(tt_ctx* c, const Complex& cx, f32** d, int32_t** verts);
// std::length_error (TT_ERR_LENGTH) with make_dense's message when the lower
// triangle of an n-point matrix exceeds the context's memory budget.
void check_dense_budget(const tt_ctx* c, u32 n);
// Non-finite coordinates of count device floats, checked without a round
// trip: settle_finite (a no-op when nothing is pending) raises the
// reference's error once the caller has enqueued its next stages.
void check_finite_async(tt_ctx* c, const f32* x, u64 count);
void settle_finite(tt_ctx* c);
// ---- tt_parse.cu
void parse_points(tt_ctx* c, const char* text, u64 bytes, f32* pts, u64 cap, u32* n, u32* dim);
void redzed_leftover(tt_ctx* c, const f32* mat, u32 n, f32 thr, unsigned long long* bits);   // tt_redzed_pred.cu

// ---- tt_assemble.cu
u64 assemble2(tt_ctx* c, const Complex& cx, const u64* keys, u64 m, const u64* piv_sorted, u64 npiv,
              u64** cidx, f32** cd, u64* napp);

// ---- tt_knn.cu
void knn_exact(tt_ctx* c, const f32* x, u32 n, u32 dim, int kind, f32 p, u32 k, u32* ids, f32* dists,
               bool defer = false);
double tc_gram_check(tt_ctx* c, u32 products, u64 seed);   // tt_knn_tc.cu
void selftest_wait_timeout(tt_ctx* c, u32 polls);           // tt_diag.cu
u64 knn_graph(tt_ctx* c, const f32* x, u32 n, u32 dim, int kind, f32 p, const u32* ids, u32 k,
              u64* rp, u32** ci, f32** w);
u64 radius_graph(tt_ctx* c, const f32* x, u32 n, u32 dim, int kind, f32 p, f32 tau, u64* rp,
                 u32** ci, f32** w);

// ---- tt_mst.cu
u64 mst_deaths(tt_ctx* c, const f32* x, u32 n, u32 dim, int kind, f32 p, f32* deaths);

}  // namespace tt
