// tt_reduce.h — the host reduction of the remaining columns (the part of the
// reference that stays sequential on the CPU).
#pragma once
#include <stdint.h>

#include <vector>

namespace tt {
namespace host {

struct Entry {
    uint64_t idx;
    float d;
};

// The complex the reducer enumerates cofacets in: a dense full matrix or a
// CSR graph (host copies), with the filtration threshold.
struct HostComplex {
    const float* mat = nullptr;   // n x n, or nullptr
    const uint64_t* rp = nullptr;
    const uint32_t* ci = nullptr;
    const float* w = nullptr;
    uint32_t n = 0;
    float thr = 0;
};

struct Bars {
    std::vector<float> birth, death;
    // critical simplices of each bar: the column's simplex (birth) and the
    // pivot (death; UINT64_MAX for essential bars)
    std::vector<uint64_t> birth_idx, death_idx;
};

struct ReduceStats {
    uint64_t columns = 0, emergent = 0;
};

// compute_pairs(dim) of the cohomology reducer. `cols` are the dimension-dim
// simplices to reduce, in descending filtration order. For dim == 1 the
// column-local part of the emergent-pair test may be supplied precomputed
// (em_idx / em_app per column, UINT64_MAX = no zero cofacet); otherwise the
// reducer evaluates it. Returns the bars; `pivots` receives the index of every
// pivot (dimension-(dim+1) simplex) found. `threads` host threads reduce
// batches of columns in parallel (0: every hardware thread); the results do
// not depend on it.
Bars compute_pairs(const HostComplex& cx, uint32_t dim, uint32_t maxdim, const std::vector<Entry>& cols,
                   const uint64_t* em_idx, const uint8_t* em_app, std::vector<uint64_t>& pivots,
                   ReduceStats& st, unsigned threads = 0);

// Reducer::assemble(dim) (rips.hpp:981-1023): the dimension-(dim + 1)
// columns — every cofacet of the dimension-dim `simplices` (any order) through
// a vertex above the simplex's largest, so each once; neither a pivot of
// dimension dim (`pivots_sorted`, ascending) nor in a zero-apparent pair —
// in descending filtration order. With `next`, every such cofacet: the
// simplices of the following dimension. *skipped receives the apparent
// count. `threads` host threads (0: all) split the simplices.
std::vector<Entry> assemble(const HostComplex& hc, uint32_t dim, uint32_t maxdim,
                            const std::vector<Entry>& simplices, const std::vector<uint64_t>& pivots_sorted,
                            std::vector<Entry>* next, uint64_t* skipped, unsigned threads = 0);

// Triangles (dimension-2 simplices with diameter <= thr) of a graph complex
// (hc.mat == nullptr), counted without storing them; the count stops soon
// after it exceeds `limit` (any value above limit then means "more").
uint64_t graph_triangles(const HostComplex& hc, uint64_t limit = UINT64_MAX);

// The same pairs and bars as compute_pairs(hc, 1, 1, cols, ...) on a graph
// complex, from the boundary matrix of its triangles instead of the
// coboundaries of its edges: essential edges are never reduced. `cols` are
// the dimension-1 columns (non-tree, non-apparent edges, descending
// filtration order); bars come out in their order, as compute_pairs emits
// them. st.emergent stays 0 (no emergent shortcut is taken). With gave_up,
// the stored reduced columns are capped at max_store entries (0: 16 a
// triangle) and the triangles at max_tris; past either cap *gave_up is set
// and nothing is returned. `threads` host threads (0: all) build and sort
// the edges and triangles; the reduction itself is sequential.
Bars graph_pairs_dim1(const HostComplex& hc, const std::vector<Entry>& cols, ReduceStats& st,
                      bool* gave_up = nullptr, uint64_t max_store = 0, uint64_t max_tris = UINT64_MAX,
                      unsigned threads = 0);

}  // namespace host
}  // namespace tt
