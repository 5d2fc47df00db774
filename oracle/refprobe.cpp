// refprobe.cpp — test infrastructure, never shipped or linked into the product.
//
// A small driver, compiled against the UNMODIFIED reference headers where they
// lie (oracle/Makefile passes their include path), that runs one front-end
// stage of the reference and dumps its raw outputs so that tests/golden can
// pin the oracle restatement and the CUDA path to the reference's own bits.
//
// Every stage reads `n * dim` little-endian float32 points from a .bin file and
// writes raw little-endian arrays to `<prefix>.<name>`:
//
//   dense   <pts> <n> <dim> <metric> <prefix>
//       .mat  n*n f32 (full layout, rips.hpp make_dense)   .encl  f32
//   dim0    <pts> <n> <dim> <metric> <threshold|inf> <prefix>
//       .eidx u64 .ed f32   sorted edges (rips.hpp Reducer::dim0 order)
//       .app  u8            zero_apparent_cofacet(edge) != none, per sorted edge
//       .cidx u64 .cd f32   dim-1 columns (descending), .h0 f32 pairs, .thr f32
//       .emg  u64 cofacet idx + f32 d + u8 flag per column (emergent probe)
//   asm     <pts> <n> <dim> <metric> <threshold|inf> <prefix>
//       dim0 + compute_pairs(1) + assemble(1):
//       .piv u64 pivot indices of dim 1, .c2idx u64 .c2d f32 dim-2 columns
//   knn     <pts> <n> <dim> <metric> <k> <prefix>     .ids u32 n*k
//   knng    <pts> <n> <dim> <metric> <k> <prefix>     .rp u64 .ci u32 .w f32
//   radius  <pts> <n> <dim> <metric> <tau> <prefix>   .rp u64 .ci u32 .w f32
//   mst     <pts> <n> <dim> <metric> <threshold|inf> <prefix>   .h0 f32 pairs
//   rzd     <pts> <n> <dim> <metric> <prefix>   dense RedZeD EdgeList (no relabel)
//       .rd f32 .rv i32 pairs
//   rzs     <pts> <n> <dim> <metric> <k> <prefix>   RedZeD EdgeList of the kNN graph
//   sdim0   <pts> <n> <dim> <metric> <k> <prefix>   Reducer::dim0 on the kNN graph
//   bars    <pts> <n> <dim> <metric> <maxdim> <prefix>   tops::persistence (dense)
//       .bars f32 triples (dim, birth, death) in canonical order
#include "turbotops/turbotops.hpp"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

using namespace tops;

namespace {

std::vector<f32> load(const char* path, u64 count) {
    std::vector<f32> x(count);
    std::ifstream in(path, std::ios::binary);
    if (!in.read(reinterpret_cast<char*>(x.data()), std::streamsize(count * 4))) {
        std::fprintf(stderr, "refprobe: short read %s\n", path);
        std::exit(2);
    }
    return x;
}

template <typename T>
void dump(const std::string& path, const T* p, u64 count) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) { std::fprintf(stderr, "refprobe: cannot write %s\n", path.c_str()); std::exit(2); }
    if (count) std::fwrite(p, sizeof(T), count, f);
    std::fclose(f);
}

f32 parse_thr(const char* s) { return std::string(s) == "inf" ? INFINITY : std::strtof(s, nullptr); }

using R = rips::Reducer<u64, rips::DenseComplex>;
using RS = rips::Reducer<u64, rips::SparseComplex>;

template <typename Red>
void dump_dim0(Red& r, const std::string& pre, f32 thr) {
    // r.dim0() ran with maxdim >= 2, so r.simplices holds every kept edge in
    // filtration order.
    std::vector<u64> eidx, cidx;
    std::vector<f32> ed, cd, h0;
    std::vector<u8> app;
    for (auto& e : r.simplices) {
        eidx.push_back(e.idx);
        ed.push_back(e.d);
        app.push_back(r.zero_apparent_cofacet(e, 2).idx != rips::kNone<u64>);
    }
    for (auto& e : r.columns) { cidx.push_back(e.idx); cd.push_back(e.d); }
    for (u64 i = 0; i < r.out.birth[0].size(); ++i) {
        h0.push_back(r.out.birth[0][i]);
        h0.push_back(r.out.death[0][i]);
    }
    // Emergent probe (rips.hpp compute_pairs, the column-local part of the
    // emergent-pair shortcut): first cofacet in descending order whose
    // diameter equals the column's, and whether it has a zero-apparent facet.
    std::vector<u64> emi;
    std::vector<f32> emd;
    std::vector<u8> emf;
    for (auto& col : r.columns) {
        u32 vd[32], cv[32];
        r.decode(col.idx, 2, vd);
        auto cf = r.zero_pivot_cofacet_v(vd, 2, col.d, cv);
        emi.push_back(cf.idx);
        emd.push_back(cf.d);
        emf.push_back(cf.idx != rips::kNone<u64> &&
                      r.zero_apparent_facet(cf, 3).idx != rips::kNone<u64>);
    }
    dump(pre + ".eidx", eidx.data(), eidx.size());
    dump(pre + ".ed", ed.data(), ed.size());
    dump(pre + ".app", app.data(), app.size());
    dump(pre + ".cidx", cidx.data(), cidx.size());
    dump(pre + ".cd", cd.data(), cd.size());
    dump(pre + ".h0", h0.data(), h0.size());
    dump(pre + ".emi", emi.data(), emi.size());
    dump(pre + ".emd", emd.data(), emd.size());
    dump(pre + ".emf", emf.data(), emf.size());
    dump(pre + ".thr", &thr, 1);
}

void dump_csr(const CsrGraph& g, const std::string& pre) {
    dump(pre + ".rp", g.row_ptr.data(), g.row_ptr.size());
    dump(pre + ".ci", g.col_idx.data(), g.col_idx.size());
    dump(pre + ".w", g.weights.data(), g.weights.size());
}

void dump_edgelist(const redzed::detail::EdgeList& el, const std::string& pre) {
    dump(pre + ".rd", el.diam.data(), el.count);
    dump(pre + ".rv", el.verts.data(), 2 * el.count);
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 7) {
        std::fprintf(stderr, "usage: refprobe <stage> <pts.bin> <n> <dim> <metric> ... <prefix>\n");
        return 2;
    }
    const std::string stage = argv[1];
    const u32 n = u32(std::strtoul(argv[3], nullptr, 10));
    const u32 dim = u32(std::strtoul(argv[4], nullptr, 10));
    const std::vector<f32> x = load(argv[2], u64(n) * dim);
    const PointCloud c{x.data(), n, dim, Metric::parse(argv[5])};
    const std::string pre = argv[argc - 1];

    if (stage == "dense") {
        rips::DenseComplex cx = rips::make_dense(n, c);
        const f32 r = cx.enclosing_radius();
        dump(pre + ".mat", cx.mat.data(), cx.mat.size());
        dump(pre + ".encl", &r, 1);
    } else if (stage == "dim0" || stage == "asm") {
        rips::DenseComplex cx = rips::make_dense(n, c);
        const f32 t = parse_thr(argv[6]);
        cx.threshold = std::isinf(t) ? cx.enclosing_radius() : t;
        rips::Barcode out;
        rips::RipsStats st;
        R r(cx, 2, out, st);
        r.dim0();
        dump_dim0(r, pre, cx.threshold);
        if (stage == "asm") {
            r.compute_pairs(1);
            std::vector<u64> piv;
            for (u64 s = 0; s < r.pivots.keys.size(); ++s)
                if (r.pivots.keys[s] != rips::kNone<u64>) piv.push_back(r.pivots.keys[s]);
            std::sort(piv.begin(), piv.end());
            r.assemble(1);
            std::vector<u64> c2i;
            std::vector<f32> c2d;
            for (auto& e : r.columns) { c2i.push_back(e.idx); c2d.push_back(e.d); }
            dump(pre + ".piv", piv.data(), piv.size());
            dump(pre + ".c2idx", c2i.data(), c2i.size());
            dump(pre + ".c2d", c2d.data(), c2d.size());
            u64 app2 = st.apparent.size() > 1 ? st.apparent[1] : 0;
            dump(pre + ".app2n", &app2, 1);
        }
    } else if (stage == "knn") {
        const KnnLists L = knn_lists_exact(c, u32(std::strtoul(argv[6], nullptr, 10)));
        dump(pre + ".ids", L.ids.data(), L.ids.size());
    } else if (stage == "knng") {
        const KnnLists L = knn_lists_exact(c, u32(std::strtoul(argv[6], nullptr, 10)));
        dump_csr(knn_graph(c, L), pre);
    } else if (stage == "radius") {
        dump_csr(radius_graph(c, std::strtof(argv[6], nullptr)), pre);
    } else if (stage == "mst") {
        const rips::Barcode b = mst::h0(c, parse_thr(argv[6]));
        std::vector<f32> h0;
        for (u64 i = 0; i < b.birth[0].size(); ++i) { h0.push_back(b.birth[0][i]); h0.push_back(b.death[0][i]); }
        dump(pre + ".h0", h0.data(), h0.size());
    } else if (stage == "rzd") {
        rips::DenseComplex cx = rips::make_dense(n, c);
        cx.threshold = cx.enclosing_radius();
        redzed::detail::DenseGeom geo(cx);
        redzed::detail::BinomialTable bt(int(n) + 1, 3);
        redzed::detail::EdgeList el;
        redzed::detail::build_edges(geo, cx.threshold, bt, el);
        dump_edgelist(el, pre);
        dump(pre + ".thr", &cx.threshold, 1);
    } else if (stage == "rzs" || stage == "sdim0") {
        const KnnLists L = knn_lists_exact(c, u32(std::strtoul(argv[6], nullptr, 10)));
        const CsrGraph g = knn_graph(c, L);
        if (stage == "rzs") {
            redzed::detail::SparseGeom<u32> geo(g);
            redzed::detail::BinomialTable bt(int(n) + 1, 3);
            redzed::detail::EdgeList el;
            redzed::detail::build_edges(geo, INFINITY, bt, el);
            dump_edgelist(el, pre);
        } else {
            rips::SparseComplex cx(g, INFINITY);
            rips::Barcode out;
            rips::RipsStats st;
            RS r(cx, 2, out, st);
            r.dim0();
            dump_dim0(r, pre, INFINITY);
        }
    } else if (stage == "bars") {
        Options o;
        o.maxdim = u32(std::strtoul(argv[6], nullptr, 10));
        o.metric = argv[5];
        const Result res = persistence(x.data(), n, dim, o);
        std::vector<f32> t;
        for (u32 d = 0; d < res.barcode.ndims(); ++d)
            for (u64 i = 0; i < res.barcode.birth[d].size(); ++i) {
                t.push_back(f32(d));
                t.push_back(res.barcode.birth[d][i]);
                t.push_back(res.barcode.death[d][i]);
            }
        dump(pre + ".bars", t.data(), t.size());
    } else {
        std::fprintf(stderr, "refprobe: unknown stage %s\n", stage.c_str());
        return 2;
    }
    return 0;
}
