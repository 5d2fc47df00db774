// host_reduce_shim.cpp — test harness only: the product's host reduction
// (turbotops_gb300/csrc/tt_reduce.cpp, compute_pairs) behind one C entry
// point, compiled with the host compiler so the CPU tests can check it
// against the reference's diagrams without a GPU. The columns it reduces come
// from the oracle's dim0 / emergent / assemble restatements.
#include <stdint.h>

#include <exception>
#include <vector>

#include "../turbotops_gb300/csrc/tt_reduce.h"

// Reduces `ncols` dimension-`dim` columns (descending filtration order) over a
// dense full matrix (rp == NULL) or a CSR graph. em_idx / em_app may be NULL
// (the emergent test then runs on the host). Bars go to birth/death (at most
// ncols each), pivots (ascending) to piv (at most ncols). Returns 0, or -1 on
// an exception.
// Host threads compute_pairs may use (0: every hardware thread).
static unsigned g_threads = 0;
extern "C" void hr_set_threads(unsigned t) { g_threads = t; }

extern "C" int hr_compute_pairs(const float* mat, const uint64_t* rp, const uint32_t* ci, const float* w, uint32_t n,
                                float thr, uint32_t dim, uint32_t maxdim, const uint64_t* cidx, const float* cd,
                                uint64_t ncols, const uint64_t* em_idx, const uint8_t* em_app, float* birth,
                                float* death, uint64_t* nbars, uint64_t* piv, uint64_t* npiv, uint64_t* emergent) {
    try {
        tt::host::HostComplex hc;
        hc.mat = mat;
        hc.rp = rp;
        hc.ci = ci;
        hc.w = w;
        hc.n = n;
        hc.thr = thr;
        std::vector<tt::host::Entry> cols(ncols);
        for (uint64_t i = 0; i < ncols; ++i) cols[i] = tt::host::Entry{cidx[i], cd[i]};
        std::vector<uint64_t> pv;
        tt::host::ReduceStats st;
        const tt::host::Bars b = tt::host::compute_pairs(hc, dim, maxdim, cols, em_idx, em_app, pv, st, g_threads);
        for (size_t i = 0; i < b.birth.size(); ++i) {
            birth[i] = b.birth[i];
            death[i] = b.death[i];
        }
        *nbars = b.birth.size();
        for (size_t i = 0; i < pv.size(); ++i) piv[i] = pv[i];
        *npiv = pv.size();
        *emergent = st.emergent;
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

// graph_pairs_dim1 (the boundary reduction of a graph complex's triangles)
// behind the same outputs as hr_compute_pairs for dimension 1; also returns
// the triangle count.
extern "C" int hr_graph_pairs_dim1(const uint64_t* rp, const uint32_t* ci, const float* w, uint32_t n, float thr,
                                   const uint64_t* cidx, const float* cd, uint64_t ncols, float* birth,
                                   float* death, uint64_t* bidx, uint64_t* didx, uint64_t* nbars,
                                   uint64_t* ntri) {
    try {
        tt::host::HostComplex hc;
        hc.rp = rp;
        hc.ci = ci;
        hc.w = w;
        hc.n = n;
        hc.thr = thr;
        std::vector<tt::host::Entry> cols(ncols);
        for (uint64_t i = 0; i < ncols; ++i) cols[i] = tt::host::Entry{cidx[i], cd[i]};
        tt::host::ReduceStats st;
        const tt::host::Bars b = tt::host::graph_pairs_dim1(hc, cols, st);
        for (size_t i = 0; i < b.birth.size(); ++i) {
            birth[i] = b.birth[i];
            death[i] = b.death[i];
            bidx[i] = b.birth_idx[i];
            didx[i] = b.death_idx[i];
        }
        *nbars = b.birth.size();
        *ntri = tt::host::graph_triangles(hc);
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

// graph_pairs_dim1 with its store capped at max_store entries: returns 1 when
// it gave up (nothing written), 0 with the bars otherwise.
extern "C" int hr_graph_pairs_dim1_capped(const uint64_t* rp, const uint32_t* ci, const float* w, uint32_t n,
                                          float thr, const uint64_t* cidx, const float* cd, uint64_t ncols,
                                          uint64_t max_store, float* birth, float* death, uint64_t* nbars) {
    try {
        tt::host::HostComplex hc;
        hc.rp = rp;
        hc.ci = ci;
        hc.w = w;
        hc.n = n;
        hc.thr = thr;
        std::vector<tt::host::Entry> cols(ncols);
        for (uint64_t i = 0; i < ncols; ++i) cols[i] = tt::host::Entry{cidx[i], cd[i]};
        tt::host::ReduceStats st;
        bool gave_up = false;
        const tt::host::Bars b = tt::host::graph_pairs_dim1(hc, cols, st, &gave_up, max_store);
        if (gave_up) return 1;
        for (size_t i = 0; i < b.birth.size(); ++i) {
            birth[i] = b.birth[i];
            death[i] = b.death[i];
        }
        *nbars = b.birth.size();
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

// The host assemble (tt_reduce.cpp assemble): the dimension-(dim + 1) columns
// of `ns` dimension-dim simplices minus the ascending pivots; with nidx !=
// NULL also every cofacet (the next dimension's simplices). Returns 0, -1 on
// an exception, -2 when a buffer is too small (counts still written).
extern "C" int hr_assemble(const float* mat, const uint64_t* rp, const uint32_t* ci, const float* w, uint32_t n,
                           float thr, uint32_t dim, uint32_t maxdim, const uint64_t* sidx, const float* sd,
                           uint64_t ns, const uint64_t* piv, uint64_t npiv, uint64_t* cidx, float* cd, uint64_t cap,
                           uint64_t* ncols, uint64_t* nidx, float* nd, uint64_t ncap, uint64_t* nnext,
                           uint64_t* napp) {
    try {
        tt::host::HostComplex hc;
        hc.mat = mat;
        hc.rp = rp;
        hc.ci = ci;
        hc.w = w;
        hc.n = n;
        hc.thr = thr;
        std::vector<tt::host::Entry> simp(ns);
        for (uint64_t i = 0; i < ns; ++i) simp[i] = tt::host::Entry{sidx[i], sd[i]};
        std::vector<uint64_t> pv(piv, piv + npiv);
        std::vector<tt::host::Entry> next;
        uint64_t skipped = 0;
        const std::vector<tt::host::Entry> cols =
            tt::host::assemble(hc, dim, maxdim, simp, pv, nidx ? &next : nullptr, &skipped, g_threads);
        *ncols = cols.size();
        *nnext = next.size();
        *napp = skipped;
        if (cols.size() > cap || next.size() > ncap) return -2;
        for (size_t i = 0; i < cols.size(); ++i) {
            cidx[i] = cols[i].idx;
            cd[i] = cols[i].d;
        }
        for (size_t i = 0; i < next.size(); ++i) {
            nidx[i] = next[i].idx;
            nd[i] = next[i].d;
        }
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}
