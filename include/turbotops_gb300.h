/* turbotops_gb300.h — C-ABI of the GB300 front end of turbotops.
 *
 * Plain C: no exceptions, no C++ or torch types cross this boundary. Every
 * entry point returns a TT_* status; tt_last_error() holds the message. The
 * C++ glue (include/turbotops_gb300.hpp) maps statuses back to the exception
 * types and messages the reference throws (std::invalid_argument,
 * std::overflow_error, std::length_error).
 *
 * Pointers named *_dev are device pointers; they are used in stream order on
 * the context's stream. Entry points ending in _h take host pointers and
 * synchronise before returning. Device results owned by the context (the
 * tt_*_out structs) stay valid until the next call on the same context.
 *
 * Reference interfaces each entry point replaces are cited as
 * file:line in dnbaker/turbotops v0.1.0.
 */
#ifndef TURBOTOPS_GB300_H
#define TURBOTOPS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TT_OK 0
#define TT_ERR_INVALID 1   /* std::invalid_argument */
#define TT_ERR_OVERFLOW 2  /* std::overflow_error */
#define TT_ERR_LENGTH 3    /* std::length_error (memory, capacity) */
#define TT_ERR_CUDA 4      /* CUDA runtime error */
#define TT_ERR_TIMEOUT 5   /* a bounded device wait ran out */
#define TT_ERR_INTERNAL 6

#define TT_METRIC_L1 0
#define TT_METRIC_L2 1
#define TT_METRIC_LINF 2
#define TT_METRIC_LP 3

typedef struct tt_ctx tt_ctx;

/* Library version, "MAJOR.MINOR.PATCH" of the reference it mirrors. */
const char* tt_version(void);

/* Context: device, stream (a cudaStream_t used as given; NULL is the legacy
 * default stream), reusable device arena. */
int tt_ctx_create(int device, void* stream, tt_ctx** out);
void tt_ctx_destroy(tt_ctx* ctx);
const char* tt_last_error(const tt_ctx* ctx);
/* Kernels launched through the context since creation. */
uint64_t tt_ctx_launches(const tt_ctx* ctx);
int tt_ctx_synchronize(tt_ctx* ctx);
/* Exact-kNN engine: 0 = automatic (the tcgen05 tensor-core Gram filter for
 * L2 in R^32 with k <= 16 and n >= 1024, else the exhaustive scan),
 * 1 = always the exhaustive scan, 2 = the filter wherever it applies.
 * Every engine returns the same lists. */
int tt_ctx_set_knn_mode(tt_ctx* ctx, int mode);
/* Options::memory_budget (turbotops.hpp:81, rips.hpp:383-416): the bytes a
 * dense distance matrix may take; 0 = half of the host's physical memory.
 * The dense entry points (tt_persistence_h with a full graph and an infinite
 * threshold, tt_dense_front_h, tt_dense_redzed_h) return TT_ERR_LENGTH with
 * make_dense's message when even the lower triangle, n(n-1)/2 floats, exceeds
 * it. It never changes a result. */
int tt_ctx_set_memory_budget(tt_ctx* ctx, uint64_t bytes);
/* Exact distance evaluations the last filtered kNN let through. */
uint64_t tt_ctx_filter_evals(const tt_ctx* ctx);
/* Candidate tiles (128 x 128 Gram blocks) the last filtered kNN computed;
 * the exhaustive product is ceil(n / 128)^2. */
uint64_t tt_ctx_filter_tiles(const tt_ctx* ctx);
/* Diagnostic, no reference counterpart: the tensor-core Gram filter's one
 * hardware assumption, measured. Runs `products` seeded 128 x 128 TF32
 * products (TF32-exact operands, the filter's augmentation step) and stores
 * the largest |D - exact| / (|a|^2 + |b|^2); the filter's margins hold while
 * it stays below 2^-19. */
int tt_tc_gram_check(tt_ctx* ctx, uint32_t products, uint64_t seed, double* max_rel);
/* Failure detection, no reference counterpart. tt_selftest_wait_timeout
 * launches one kernel whose mbarrier wait nobody completes, bounded by
 * `polls` (1 .. 2^20) polls: the wait runs out, the kernel records it in its
 * error word and ends normally, and the call returns TT_ERR_TIMEOUT — the
 * path every bounded wait in the library takes — leaving the context usable.
 * tt_ctx_inject_alloc_failure makes the nth next device-arena allocation of
 * the context fail as if cudaMalloc had (host-side injection, no device
 * call): that call returns TT_ERR_LENGTH ("device memory exhausted"). */
int tt_selftest_wait_timeout(tt_ctx* ctx, uint32_t polls);
int tt_ctx_inject_alloc_failure(tt_ctx* ctx, uint32_t nth);
/* Stream-ordered copy of bytes between any two device or host addresses
 * (lets bindings move context-owned results into their own buffers). */
int tt_copy_async(tt_ctx* ctx, void* dst, const void* src, size_t bytes);

/* Metric::parse + Metric::minkowski (metric.hpp:227-253): "l1" | "l2" |
 * "linf" | "euclidean" | "manhattan" | "chebyshev" | "lp:<p>", p >= 1. */
int tt_metric_parse(const char* s, int* kind, float* p);

/* make_dense, full layout (rips.hpp:391-403) + enclosing_radius
 * (rips.hpp:370-380). x_dev: n x dim row-major; mat_dev: n x n.
 * *enclosing (host, may be NULL) receives min_i max_j d(i, j) (+inf if n = 0). */
int tt_dense_distances(tt_ctx* ctx, const float* x_dev, uint32_t n, uint32_t dim, int kind, float p,
                       float* mat_dev, float* enclosing);

/* No counterpart in the reference. tt_dense_distances for callers that
 * cannot allocate device memory during the call (all device memory already
 * handed to their own pool, or a loop that must not take the
 * synchronisation cudaMalloc/cudaFree imply): no context, no cudaMalloc,
 * cudaFree or allocating library call. The per-row maxima live in a fixed
 * 1 MiB array in the library's device memory, so n <= 262144 (larger n
 * returns TT_ERR_LENGTH before any work). Outputs: mat_dev (n x n) and
 * radius_dev (one float, device memory), in stream order on `stream`
 * (cudaStream_t; NULL = legacy default stream) of the current device.
 * The first call on each device loads the library's module there (make it
 * before any stream capture). All calls on a device share the array; calls
 * that overlap on the GPU race and must be serialised by the caller.
 * Errors: tt_last_error(NULL). */
int tt_dense_distances_static(const float* x_dev, uint32_t n, uint32_t dim, int kind, float p, float* mat_dev,
                              float* radius_dev, void* stream);

/* Result of tt_dim0: device arrays owned by the context. */
typedef struct tt_dim0_out {
    uint64_t edges;                     /* kept edges (d <= threshold) */
    const uint64_t* edge_keys_dev;      /* sorted: diameter bits << 33 | (2^33-1 - index) */
    const uint8_t* apparent_dev;        /* per sorted edge: zero-apparent (maxdim >= 1) */
    const uint8_t* tree_dev;            /* per sorted edge: in the spanning forest */
    uint64_t columns;                   /* dim-1 columns, descending filtration order */
    const uint64_t* col_index_dev;
    const float* col_diameter_dev;
    const uint64_t* col_cofacet_dev;    /* first zero cofacet (triangle index) or UINT64_MAX */
    const uint8_t* col_cofacet_app_dev; /* that cofacet has a zero-apparent facet */
    uint64_t h0_finite;                 /* finite H0 bars with death > 0, discovery order */
    const float* h0_death_dev;
    uint64_t essential;                 /* connected components: essential H0 bars */
} tt_dim0_out;

/* Reducer::dim0 (rips.hpp:685-870). The complex is the dense full matrix
 * mat_dev (n x n) when it is not NULL, else the CSR graph rp/ci/w (device;
 * CsrGraph layout core.hpp:92-98, rows sorted by neighbour id). Edges with
 * d <= threshold are kept. maxdim >= 1 computes apparent flags and columns.
 * n <= 131072 (edge indices must fit the packed keys' 33-bit field; the
 * host-buffer entry points and tt_persistence_h take larger complexes). */
int tt_dim0(tt_ctx* ctx, const float* mat_dev, const uint64_t* rp_dev, const uint32_t* ci_dev,
            const float* w_dev, uint32_t n, float threshold, uint32_t maxdim, tt_dim0_out* out);

/* redzed::detail::build_edges (redzed.hpp:545-613): kept edges sorted by
 * (diameter asc, combinatorial index asc); verts_dev holds (i, j), i < j.
 * Same complex convention as tt_dim0. *count receives the edge count;
 * TT_ERR_LENGTH if it exceeds cap (nothing written). */
int tt_redzed_edges(tt_ctx* ctx, const float* mat_dev, const uint64_t* rp_dev, const uint32_t* ci_dev,
                    const float* w_dev, uint32_t n, float threshold, float* diam_dev, int32_t* verts_dev,
                    uint64_t cap, uint64_t* count);

/* knn_lists_exact (graph.hpp:211-225): the k nearest neighbours of every
 * point, ascending by (distance, id), self excluded; k is clamped to n - 1
 * (the row stride of ids_dev / dists_dev is the clamped k, *k_out). k <= 32.
 * dists_dev may be NULL. */
int tt_knn(tt_ctx* ctx, const float* x_dev, uint32_t n, uint32_t dim, int kind, float p, uint32_t k,
           uint32_t* ids_dev, float* dists_dev, uint32_t* k_out);

/* Result of a graph builder: a CsrGraph (core.hpp:92-98) with device arrays
 * owned by the context; row_ptr_dev has n + 1 entries. */
typedef struct tt_csr_out {
    uint32_t n;
    uint64_t nnz;              /* 2m */
    const uint64_t* row_ptr_dev;
    const uint32_t* col_dev;
    const float* weight_dev;
} tt_csr_out;

/* knn_lists_exact + knn_graph (graph.hpp:211-225, :286-304): the symmetric
 * kNN graph, rows sorted by neighbour id, weights d(i, j). A non-finite
 * coordinate is TT_ERR_INVALID ("persistence: non-finite coordinate"), as
 * for PointCloud; it is checked on the device. */
int tt_knn_graph(tt_ctx* ctx, const float* x_dev, uint32_t n, uint32_t dim, int kind, float p, uint32_t k,
                 tt_csr_out* out);

/* radius_graph (graph.hpp:170-201): all pairs with d <= tau. */
int tt_radius_graph(tt_ctx* ctx, const float* x_dev, uint32_t n, uint32_t dim, int kind, float p, float tau,
                    tt_csr_out* out);

/* mst::h0 (mst.hpp:25-99): the n - 1 minimum-spanning-tree weights of the
 * complete graph, ascending, into deaths_dev (capacity n). The reference's
 * bars follow: deaths > threshold add essential classes, deaths > 0 are
 * finite bars. Non-finite coordinates: TT_ERR_INVALID, as tt_knn_graph. */
int tt_mst_deaths(tt_ctx* ctx, const float* x_dev, uint32_t n, uint32_t dim, int kind, float p, float* deaths_dev);

/* Host-buffer form of tt_knn_graph (what the reference's
 * knn_lists_exact + knn_graph front end binds): points in, CsrGraph out.
 * row_ptr_h has n + 1 entries; col_h / weight_h hold up to cap entries
 * (TT_ERR_LENGTH beyond, *nnz always set). */
int tt_knn_graph_h(tt_ctx* ctx, const float* x_h, uint32_t n, uint32_t dim, int kind, float p, uint32_t k,
                   uint64_t* row_ptr_h, uint32_t* col_h, float* weight_h, uint64_t cap, uint64_t* nnz);
/* Host-buffer form of tt_radius_graph (radius_graph, graph.hpp:170-201):
 * points and tau in, the CsrGraph of the pairs with d <= tau out; capacities
 * as in tt_knn_graph_h (a first call with cap = 0 returns the count). */
int tt_radius_graph_h(tt_ctx* ctx, const float* x_h, uint32_t n, uint32_t dim, int kind, float p, float tau,
                      uint64_t* row_ptr_h, uint32_t* col_h, float* weight_h, uint64_t cap, uint64_t* nnz);

/* Device results of the kNN flag-complex front end: the graph plus dim0. */
typedef struct tt_knn_front_out {
    tt_csr_out graph;
    tt_dim0_out dim0;
} tt_knn_front_out;

/* knn_lists_exact -> knn_graph -> Reducer::dim0 of rips::compute_graph
 * (turbotops.hpp:260-298, threshold +inf), all on the device. n <= 131072
 * (packed edge keys, as tt_dim0); tt_knn_front_h takes any n. Non-finite
 * coordinates: TT_ERR_INVALID, as tt_knn_graph. */
int tt_knn_front(tt_ctx* ctx, const float* x_dev, uint32_t n, uint32_t dim, int kind, float p, uint32_t k,
                 uint32_t maxdim, tt_knn_front_out* out);

/* Front end of the kNN flag-complex path with host buffers (what
 * persistence(points, ...) with graph = knn binds, turbotops.hpp:260-298:
 * knn_lists_exact -> knn_graph -> Reducer::dim0 of rips::compute_graph):
 * points in; the CsrGraph, the H0 deaths, the essential count and the dim-1
 * columns (+ emergent probe) out. Capacities as in tt_knn_graph_h and
 * tt_dense_front_h; every count is always written. */
int tt_knn_front_h(tt_ctx* ctx, const float* x_h, uint32_t n, uint32_t dim, int kind, float p, uint32_t k,
                   uint32_t maxdim, uint64_t* row_ptr_h, uint32_t* col_h, float* weight_h, uint64_t cap,
                   uint64_t* nnz, float* h0_h, uint64_t* nh0, uint64_t* essential, uint64_t* col_idx_h,
                   float* col_d_h, uint64_t* col_cf_h, uint8_t* col_cf_app_h, uint64_t col_cap, uint64_t* ncols,
                   uint64_t* nedges);

/* Front end of the dense full-Rips path with host buffers (the call the
 * reference's rips::compute_dense front end binds, rips.hpp:1068-1075 +
 * :685-870): points -> distances -> enclosing radius -> dim0, everything a
 * host reducer needs, copied back.
 *   mat_h      n x n distances (may be NULL)
 *   h0_h       finite H0 deaths (capacity n)
 *   col_idx_h / col_d_h / col_cf_h / col_cf_app_h   columns (capacity n(n-1)/2
 *              or *ncols from a first call with col_idx_h == NULL)
 *   thr_inout  threshold in (+inf: enclosing radius), effective threshold out */
int tt_dense_front_h(tt_ctx* ctx, const float* x_h, uint32_t n, uint32_t dim, int kind, float p,
                     uint32_t maxdim, float* thr_inout, float* mat_h, float* h0_h, uint64_t* nh0,
                     uint64_t* essential, uint64_t* col_idx_h, float* col_d_h, uint64_t* col_cf_h,
                     uint8_t* col_cf_app_h, uint64_t col_cap, uint64_t* ncols, uint64_t* nedges);

/* RedZeD front ends with host buffers: what redzed::detail::Engine::run
 * (redzed.hpp:1316-1408) reads before its reduction — make_dense +
 * enclosing_radius (rips.hpp:370-416) and build_edges (redzed.hpp:545-613)
 * for dense full Rips, build_edges over a weighted graph (SparseGeom) — so
 * the reference's RedZeD engine can run on the host from what the GPU built.
 *   tt_dense_redzed_h: points -> the n x n matrix (mat_h, may be NULL), the
 *     threshold (thr_inout: +inf in, the enclosing radius out) and the edges
 *     with d <= threshold in (d asc, combinatorial index asc) order,
 *     vertices i < j (diam_h: count floats, verts_h: 2 count ints).
 *   tt_graph_redzed_h: host CSR (row_ptr n + 1, 2m columns and weights, rows
 *     sorted by id) -> its edges with w <= threshold in the same order.
 * *count always receives the edge count; TT_ERR_LENGTH when it exceeds cap
 * (nothing copied: call again with a larger buffer). */
int tt_dense_redzed_h(tt_ctx* ctx, const float* x_h, uint32_t n, uint32_t dim, int kind, float p, float* thr_inout,
                      float* mat_h, float* diam_h, int32_t* verts_h, uint64_t cap, uint64_t* count);
/* tt_dense_redzed_h plus RedZeD's static leftover-coface predicate
 * (redzed.hpp:1238-1273, :728-765, :1193-1202) for every kept edge, computed
 * on the GPU: leftover_h (n x ceil(n / 64) words, row u, bit v for u < v) has
 * bit (u, v) set when some w != u, v has d(u, w) <= d(u, v) and d(v, w) <=
 * d(u, v) and makes {u, v, w} ready (w < u; u < w < v with d(w, v) < d(u, v);
 * w > v with both strictly shorter) — what the engine's
 * has_leftover_coface answers for that edge when its active enumeration
 * excluded no vertex. */
int tt_dense_redzed_pred_h(tt_ctx* ctx, const float* x_h, uint32_t n, uint32_t dim, int kind, float p,
                           float* thr_inout, float* mat_h, float* diam_h, int32_t* verts_h, uint64_t cap,
                           uint64_t* count, uint64_t* leftover_h);
/* The same predicate bits for a full n x n matrix already on the device
 * (mat_dev, e.g. one cloud of a batch, tt_batch_out.mats_dev) cut at thr. */
int tt_redzed_leftover_h(tt_ctx* ctx, const float* mat_dev, uint32_t n, float threshold, uint64_t* leftover_h);
int tt_graph_redzed_h(tt_ctx* ctx, const uint64_t* row_ptr_h, const uint32_t* col_h, const float* weight_h,
                      uint32_t n, float threshold, float* diam_h, int32_t* verts_h, uint64_t cap, uint64_t* count);

/* Reducer::assemble(1) (rips.hpp:981-1023) over the dense matrix mat_dev:
 * the dimension-2 columns generated from the sorted kept edges
 * (edge_keys_dev, m Ripser keys as tt_dim0 returns them), minus the
 * dimension-1 pivots (pivots_dev, npiv triangle indices, any order) and the
 * triangles in zero-apparent pairs, in descending filtration order.
 * *columns receives the count; *col_index_dev / *col_diameter_dev point at
 * context-owned arrays; *apparent receives the skipped-apparent count.
 * Requires C(n, 3) < 2^33. */
int tt_assemble(tt_ctx* ctx, const float* mat_dev, uint32_t n, float threshold, const uint64_t* edge_keys_dev,
                uint64_t m, const uint64_t* pivots_dev, uint64_t npiv, uint64_t* columns,
                const uint64_t** col_index_dev, const float** col_diameter_dev, uint64_t* apparent);

/* ---- Batched dense front end, replayed from a captured CUDA graph ----
 * The front end the reference runs per full-Rips cloud (turbotops.hpp:230-259
 * with RedZeD: make_dense, enclosing_radius, build_edges) for a whole batch of
 * clouds of uneven size in one pass: a persistent work-queue kernel over every
 * cloud's distance tiles, per-cloud enclosing radii, and one sort of all
 * clouds' kept edges. Buffers are sized for the worst case at creation, so a
 * run has no host round trip and (use_graph != 0) is one graph launch. */
typedef struct tt_batch tt_batch;
typedef struct tt_batch_out {
    uint32_t clouds;
    uint64_t total_points;
    const float* radius_dev;          /* per cloud: enclosing radius (the threshold) */
    const uint64_t* edge_offset_dev;  /* clouds + 1 offsets into diam/verts */
    const float* diam_dev;            /* per cloud: kept edges, (d asc, comb asc) */
    const int32_t* verts_dev;         /* (i, j) local vertex ids, i < j */
    const float* mats_dev;            /* per cloud: n x n distances, back to back */
    void* stream;                     /* the batch's own stream (cudaStream_t) */
} tt_batch_out;
/* sizes: points per cloud (host). Points go into tt_batch_points(b):
 * clouds back to back, row-major (sum of sizes) x dim float32 on the device. */
int tt_batch_create(tt_ctx* ctx, const uint32_t* sizes, uint32_t count, uint32_t dim, int kind, float p,
                    int use_graph, tt_batch** out);
float* tt_batch_points(tt_batch* b);
/* Runs the batch on its stream; wait != 0 synchronises before returning. */
int tt_batch_run(tt_batch* b, int wait);
int tt_batch_result(tt_batch* b, tt_batch_out* out);
void tt_batch_destroy(tt_batch* b);
/* The autotuner's pick, no reference counterpart: the first run of a batch
 * times every distance-tile shape on its points (the pick is cached per
 * metric, dimension and size class) and keeps the fastest. tile_rows x
 * tile_cols is the shape in use; shape_ms (room for 8) the time of each
 * candidate's pass (0 where the pick came from the cache, *from_cache = 1);
 * *shapes the number of candidates. Valid after the first tt_batch_run. */
int tt_batch_tuning(tt_batch* b, uint32_t* tile_rows, uint32_t* tile_cols, float* shape_ms, uint32_t* shapes,
                    int* from_cache);

/* ---- Differentiable persistence (no counterpart in the reference) ----
 * tt_topo_forward: for clouds stored back to back in x_dev (sizes[q] points
 * each, dim coordinates), the dense full-Rips diagram up to H1 with each bar's
 * critical edge(s), as global point ids (host arrays owned by the result;
 * release with tt_topo_free). H0: finite bars only. H1: every bar; essential
 * bars have death +inf and death edge (UINT32_MAX, UINT32_MAX). The front end
 * runs on the GPU, the column reductions of all clouds on `threads` host
 * threads (0 = all cores). */
typedef struct tt_topo_out {
    uint32_t clouds;
    const uint64_t* h0_offset;      /* clouds + 1 */
    const float* h0_death;
    const uint32_t* h0_edge;        /* 2 per bar */
    const uint64_t* h1_offset;      /* clouds + 1 */
    const float* h1_birth;
    const float* h1_death;
    const uint32_t* h1_birth_edge;  /* 2 per bar */
    const uint32_t* h1_death_edge;  /* 2 per bar */
    void* opaque;
} tt_topo_out;
int tt_topo_forward(tt_ctx* ctx, const float* x_dev, const uint32_t* sizes, uint32_t count, uint32_t dim, int kind,
                    float p, int threads, tt_topo_out** out);
void tt_topo_free(tt_topo_out* out);
/* The adjoint: grad_x_dev[u] += g_e * dd/dx_u, grad_x_dev[v] -= g_e * dd/dx_u
 * for every edge e = (u, v) of edges_dev (2 per edge, point ids) with
 * upstream gradient grad_d_dev[e], for the metric (kind, p). Accumulates
 * (float atomics) into grad_x_dev, which the caller zeroes. */
int tt_topo_adjoint(tt_ctx* ctx, const float* x_dev, uint32_t dim, int kind, float p, const uint32_t* edges_dev,
                    const float* grad_d_dev, uint64_t m, float* grad_x_dev);

/* A persistence diagram (rips.hpp Barcode :52-67) in discovery order plus the
 * reference's telemetry (turbotops.hpp Stats :85-96). Host memory owned by
 * the library: release with tt_barcode_free. */
typedef struct tt_barcode {
    uint32_t ndims;
    uint64_t total;
    uint64_t* count;     /* bars per dimension (ndims entries) */
    float* birth;        /* all bars, dimension-major, discovery order */
    float* death;        /* +inf for essential classes */
    char method[32];     /* "dense", "sparse" or "mst" */
    float threshold;     /* effective filtration cutoff */
    uint64_t edges;
    uint64_t columns[32], apparent[32], emergent[32];
} tt_barcode;

/* read_text_points (src/turbotops.cpp:126-155) on the device: the bytes of
 * a text file (text_h, a leading UTF-8 BOM skipped; one point per '\n'-ended
 * line, '#' starting a comment, separators ' ', '\t', '\v', '\f', '\r',
 * ',', ';') -> *n points of *dim float32 coordinates in pts_h (row-major, up
 * to cap floats; bytes / 2 + 1 always suffice), each the value std::strtof
 * gives the token. Decimal and "inf" tokens are converted on the GPU
 * (correctly rounded); other tokens, and decimals of more than 19 significant
 * digits that the first 19 cannot decide, by the host C library's strtof.
 * Errors (TT_ERR_INVALID), the first in file order as the reference reports
 * them: "bad coordinate '<token>'", "inconsistent row length at point N"
 * (the reference's CLI prefixes the path). */
int tt_parse_points_h(tt_ctx* ctx, const char* text_h, uint64_t bytes, float* pts_h, uint64_t cap, uint32_t* n,
                      uint32_t* dim);

/* tops::persistence(points, n, dim, Options) (turbotops.hpp:211-303) with
 * the front end on the GPU and compute_pairs on the host:
 *   knn = 0, maxdim = 0          complete-graph MST H0 (mst::h0)
 *   knn = 0, threshold = +inf    dense full Rips cut at the enclosing radius
 *   knn = 0, threshold < inf     radius graph, sparse flag complex
 *   knn = 1                      exact kNN graph (k neighbours), sparse flag complex
 * Any maxdim <= 30 (dimensions above the GPU's are assembled on the host);
 * k <= 32 and dim <= 64 for the graph scans. */
int tt_persistence_h(tt_ctx* ctx, const float* x_h, uint32_t n, uint32_t dim, int kind, float p, uint32_t maxdim,
                     float threshold, int knn, uint32_t k, tt_barcode** out);
/* tops::persistence(const CsrGraph&, maxdim, threshold, threads, mode)
 * (turbotops.hpp:179-207): the flag complex of a weighted graph given as
 * host CSR arrays (row_ptr n + 1 entries, 2m columns and weights). The graph
 * must satisfy CsrGraph::valid() (core.hpp:137-148: row_ptr[0] = 0, even
 * entry count, columns < n, no self loops, rows strictly ascending, the
 * weight of (v, u) equal to that of (u, v)); otherwise TT_ERR_INVALID with
 * the reference's message. Edges with weight <= threshold are kept. GPU
 * front end limit: maxdim <= 1. */
int tt_persistence_graph_h(tt_ctx* ctx, const uint64_t* row_ptr_h, const uint32_t* col_h, const float* weight_h,
                           uint32_t n, uint32_t maxdim, float threshold, tt_barcode** out);
void tt_barcode_free(tt_barcode* b);

#ifdef __cplusplus
}
#endif
#endif
