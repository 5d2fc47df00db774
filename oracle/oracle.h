/* oracle.h — TEST INFRASTRUCTURE ONLY: the CPU oracle of the front end.
 *
 * A plain, scalar restatement of the reference's front-end algorithms
 * (dnbaker/turbotops v0.1.0), used by tests/ and bench.py's CPU leg as the
 * checker. It is never linked into, called by, or shipped with the product
 * library (turbotops_gb300/), which fails loudly without its CUDA build.
 *
 * Parity: pinned against golden vectors dumped by the reference itself
 * (oracle/refprobe.cpp, fixtures in tests/golden) for L1, L2, L-inf and integer-p
 * Lp, on any host. For non-integer p the reference's bits depend on the host:
 * its pow01_8 takes a hardware reciprocal estimate and its scalar pow is the
 * host libm's powf. The oracle models an aarch64 host (the GB300 machine's Grace
 * CPU: FRECPE + one FRECPS step through SIMDe's NEON translation, glibc powf,
 * GCC's default contraction), aarch64_math.h, pinned against fixtures that
 * the reference built on that host dumped (the tests/golden a64 fixtures).
 *
 * Metric kinds: 0 = L1, 1 = L2, 2 = L-inf, 3 = Lp (p >= 1).
 */
#ifndef TT_ORACLE_H
#define TT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Lp model bits (oracle.cpp g_lp_model): 1 fused fnmadd in the reciprocal
 * refinement, 2 fused lg multiply-add, 4 glibc powf's aarch64 rounding of
 * y*log2(x). Default 7. */
void or_set_lp_model(int model);
int or_get_lp_model(void);
/* The modelled scalar pow (glibc powf) and SIMDe rcp_ps (FRECPE + FRECPS). */
float or_powf(float x, float y);
float or_rcp(float x);

/* kern::l1/l2/linf/lp (metric.hpp:92-207), reference lane order. */
float or_dist(int kind, float p, const float* a, const float* b, uint32_t dim);
/* make_dense full layout (rips.hpp:391-403): mat[i*n+j] = d(i,j) for i>j, mirrored. */
void or_dense(const float* x, uint32_t n, uint32_t dim, int kind, float p, float* mat);
/* DenseComplex::enclosing_radius (rips.hpp:370-380). */
float or_enclosing_radius(const float* mat, uint32_t n);

/* Reducer::dim0 (rips.hpp:685-870) over a dense full matrix (rp == NULL) or a
 * CSR graph (rp/ci/w, rows sorted by neighbour id).  Buffers are caller-sized:
 * edges <= n(n-1)/2, columns <= edges, h0 pairs <= 2n floats.
 * Returns the number of kept edges; *ncols, *nh0 receive the other counts. */
uint64_t or_dim0(const float* mat, const uint64_t* rp, const uint32_t* ci, const float* w,
                 uint32_t n, float thr, uint32_t maxdim,
                 uint64_t* eidx, float* ed, uint8_t* app,
                 uint64_t* cidx, float* cd, uint64_t* ncols, float* h0, uint64_t* nh0);

/* Column-local part of the emergent-pair shortcut (rips.hpp:903-928) for
 * dim-1 columns: first cofacet (descending) with diameter == column's, and
 * whether it has a zero-apparent facet. */
void or_emergent(const float* mat, const uint64_t* rp, const uint32_t* ci, const float* w,
                 uint32_t n, const uint64_t* cidx, const float* cd, uint64_t ncols,
                 uint64_t* cf_idx, float* cf_d, uint8_t* cf_app);

/* Reducer::assemble(1) (rips.hpp:981-1023) over a dense full matrix: the dim-2
 * columns from the sorted kept edges, minus the dim-1 pivots (sorted
 * ascending) and apparent triangles, sorted descending.  Returns the column
 * count (written up to cap); *napp receives the apparent count. */
uint64_t or_assemble(const float* mat, uint32_t n, float thr,
                     const uint64_t* sidx, const float* sd, uint64_t ns,
                     const uint64_t* piv, uint64_t npiv,
                     uint64_t* cidx, float* cd, uint64_t cap, uint64_t* napp);

/* knn_lists_exact (graph.hpp:211-225): ascending (d, id), self excluded. */
void or_knn(const float* x, uint32_t n, uint32_t dim, int kind, float p, uint32_t k, uint32_t* ids);
/* Rows [q0, q1) of the same lists on `threads` host threads. */
void or_knn_rows(const float* x, uint32_t n, uint32_t dim, int kind, float p, uint32_t k, uint32_t q0,
                 uint32_t q1, uint32_t threads, uint32_t* ids);
/* knn_graph (graph.hpp:286-304) + CsrGraph::from_rows: returns nnz; rp has n+1. */
uint64_t or_knn_graph(const float* x, uint32_t n, uint32_t dim, int kind, float p,
                      const uint32_t* ids, uint32_t k, uint64_t* rp, uint32_t* ci, float* w);
/* radius_graph (graph.hpp:170-201): returns nnz (written up to cap). */
uint64_t or_radius_graph(const float* x, uint32_t n, uint32_t dim, int kind, float p, float tau,
                         uint64_t* rp, uint32_t* ci, float* w, uint64_t cap);
/* mst::h0 (mst.hpp:25-99): bars as (birth, death) pairs; returns the bar count. */
uint64_t or_mst_h0(const float* x, uint32_t n, uint32_t dim, int kind, float p, float thr,
                   float* bars);
/* redzed::detail::build_edges (redzed.hpp:545-613): kept edges in
 * (d asc, combinatorial index asc) order, vertices (i < j). Dense full matrix
 * (rp == NULL) or CSR. Returns the edge count. */
uint64_t or_redzed_edges(const float* mat, const uint64_t* rp, const uint32_t* ci, const float* w,
                         uint32_t n, float thr, float* d, int32_t* verts);

#ifdef __cplusplus
}
#endif
#endif
