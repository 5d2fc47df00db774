// refbench.cpp — test and benchmark infrastructure, never shipped or linked
// into the product.
//
// Times the UNMODIFIED reference (compiled against its own headers by
// oracle/Makefile, with the reference Makefile's default flags) on the host
// cores, through the reference's own public functions, and prints one JSON line
// with the seconds of every timed step and of each phase.
//
//   refbench <stage> <pts.bin> <n> <dim> <metric> <k> <maxdim> <warmup> <steps> <threads>
//
// stages
//   knnfront   the front end of the symmetric kNN flag complex, as
//              tops::persistence runs it on the coboundary engine
//              (turbotops.hpp:263-280, rips.hpp:1038-1083): knn_lists_exact
//              (graph.hpp:211) -> knn_graph (graph.hpp:286) ->
//              Reducer<u64, SparseComplex>::dim0 (rips.hpp:685), i.e. the
//              sorted kept edges, apparent pairs, H0 and the dim-1 columns
//   knnwhole   tops::persistence(points, Options{graph = Knn, k, maxdim})
//              (turbotops.hpp:211): the whole diagram, mode auto
//   dense      tops::persistence(points, Options{graph = Full, maxdim}):
//              the whole full-Rips diagram cut at the enclosing radius
//   mst        mst::h0 (mst.hpp:25): complete-graph H0, the maxdim 0 path
//   knnlists   knn_lists_exact alone
//
// threads = 0 uses every hardware thread (the reference's default).
#include "turbotops/turbotops.hpp"

#include <chrono>
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
        std::fprintf(stderr, "refbench: short read %s\n", path);
        std::exit(2);
    }
    return x;
}

double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Phases {
    std::vector<std::string> names;
    std::vector<double> secs;
    void add(const char* n, double s) {
        for (size_t i = 0; i < names.size(); ++i)
            if (names[i] == n) { secs[i] += s; return; }
        names.push_back(n);
        secs.push_back(s);
    }
};

}  // namespace

int main(int argc, char** argv) {
    if (argc != 11) {
        std::fprintf(stderr,
                     "usage: refbench <stage> <pts.bin> <n> <dim> <metric> <k> <maxdim> <warmup> <steps> "
                     "<threads>\n");
        return 2;
    }
    const std::string stage = argv[1];
    const u32 n = u32(std::strtoul(argv[3], nullptr, 10));
    const u32 dim = u32(std::strtoul(argv[4], nullptr, 10));
    const std::string metric = argv[5];
    const u32 k = u32(std::strtoul(argv[6], nullptr, 10));
    const u32 maxdim = u32(std::strtoul(argv[7], nullptr, 10));
    const int warmup = std::atoi(argv[8]);
    const int steps = std::atoi(argv[9]);
    const u32 threads = u32(std::strtoul(argv[10], nullptr, 10));
    if (threads) set_num_threads(threads);
    const std::vector<f32> x = load(argv[2], u64(n) * dim);
    const PointCloud c{x.data(), n, dim, Metric::parse(metric)};

    Phases ph;
    std::vector<double> step_s;
    u64 check = 0;   // a count from each step's output, so nothing is optimised away
    for (int it = 0; it < warmup + steps; ++it) {
        Phases cur;
        const double t0 = now();
        if (stage == "knnfront") {
            double a = now();
            const KnnLists L = knn_lists_exact(c, k);
            cur.add("knn_s", now() - a);
            a = now();
            const CsrGraph g = knn_graph(c, L);
            cur.add("graph_s", now() - a);
            a = now();
            rips::SparseComplex cx(g, INFINITY);
            rips::Barcode out;
            out.ensure(maxdim);
            rips::RipsStats st;
            rips::Reducer<u64, rips::SparseComplex> r(cx, maxdim, out, st);
            r.dim0();
            cur.add("dim0_s", now() - a);
            check = r.columns.size() + out.birth[0].size();
        } else if (stage == "knnlists") {
            const KnnLists L = knn_lists_exact(c, k);
            check = L.ids.size();
        } else if (stage == "knnwhole" || stage == "dense") {
            Options o;
            o.maxdim = maxdim;
            o.metric = metric;
            o.graph = stage == "knnwhole" ? Options::Graph::Knn : Options::Graph::Full;
            o.k = k;
            const Result res = persistence(x.data(), n, dim, o);
            check = 0;
            for (u32 d = 0; d < res.barcode.ndims(); ++d) check += res.barcode.birth[d].size();
            cur.add("graph_s", res.stats.seconds_graph);
        } else if (stage == "mst") {
            const rips::Barcode b = mst::h0(c, INFINITY);
            check = b.birth[0].size();
        } else {
            std::fprintf(stderr, "refbench: unknown stage %s\n", stage.c_str());
            return 2;
        }
        const double s = now() - t0;
        if (it >= warmup) {
            step_s.push_back(s);
            for (size_t i = 0; i < cur.names.size(); ++i) ph.add(cur.names[i].c_str(), cur.secs[i]);
        }
    }
    std::printf("{\"stage\": \"%s\", \"threads\": %u, \"check\": %llu, \"steps_s\": [", stage.c_str(),
                num_threads(), (unsigned long long)check);
    for (size_t i = 0; i < step_s.size(); ++i) std::printf("%s%.6f", i ? ", " : "", step_s[i]);
    std::printf("], \"phases_s\": {");
    for (size_t i = 0; i < ph.names.size(); ++i)
        std::printf("%s\"%s\": %.6f", i ? ", " : "", ph.names[i].c_str(), ph.secs[i] / (steps ? steps : 1));
    std::printf("}}\n");
    return 0;
}
