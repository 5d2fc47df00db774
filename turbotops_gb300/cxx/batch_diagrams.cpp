// batch_diagrams.cpp — whole diagrams of a batch of dense full-Rips clouds
// through the C++ drop-in (include/turbotops_gb300.hpp, compiled inside the
// reference's include tree, as a user of the reference's C++ API would):
// tops::gb300::persistence_batch (one batched GPU front end, then the
// reference's RedZeD engine per cloud on the host threads) against the
// reference's own tops::persistence called once per cloud, as its users do.
//
//   batch_diagrams <clouds.bin> <metric> <maxdim> <reps> <ref_stride> <threads>
//
// clouds.bin: u32 count, u32 dim, count x u32 sizes, then the points (float32,
// row-major, clouds back to back). Every ref_stride-th cloud (0: none) is
// also computed by tops::persistence; its canonical diagram must equal the
// batch's. The batch runs once more with the engine's own leftover-coface
// scan instead of the device's predicate: same bars, same order. Prints one JSON line: the batch's seconds per run (front end, host
// copies, reductions), the reference's seconds for the compared clouds, and
// whether every compared diagram was identical.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "turbotops_gb300.hpp"

using namespace tops;

namespace {

std::vector<std::pair<u32, u32>> canon(const rips::Barcode& b, u32 d) {
    std::vector<std::pair<u32, u32>> v;
    if (d >= b.ndims()) return v;
    for (u64 i = 0; i < b.birth[d].size(); ++i) {
        u32 x, y;
        std::memcpy(&x, &b.birth[d][i], 4);
        std::memcpy(&y, &b.death[d][i], 4);
        v.emplace_back(x, y);
    }
    std::sort(v.begin(), v.end());
    return v;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 7) {
        std::fprintf(stderr, "usage: batch_diagrams <clouds.bin> <metric> <maxdim> <reps> <ref_stride> <threads>\n");
        return 2;
    }
    std::ifstream in(argv[1], std::ios::binary);
    u32 count = 0, dim = 0;
    in.read(reinterpret_cast<char*>(&count), 4);
    in.read(reinterpret_cast<char*>(&dim), 4);
    std::vector<u32> sizes(count);
    in.read(reinterpret_cast<char*>(sizes.data()), 4 * std::streamsize(count));
    u64 total = 0;
    for (u32 s : sizes) total += s;
    std::vector<f32> pts(total * dim);
    if (!in.read(reinterpret_cast<char*>(pts.data()), std::streamsize(4 * pts.size()))) {
        std::fprintf(stderr, "batch_diagrams: short read\n");
        return 2;
    }
    std::vector<const f32*> clouds(count);
    for (u64 q = 0, at = 0; q < count; at += sizes[q], ++q) clouds[q] = pts.data() + at * dim;
    Options o;
    o.metric = argv[2];
    o.maxdim = u32(std::stoul(argv[3]));
    const int reps = std::stoi(argv[4]);
    const u32 stride = u32(std::stoul(argv[5]));
    const u32 threads = u32(std::stoul(argv[6]));

    using clk = std::chrono::steady_clock;
    std::vector<Result> res;
    gb300::persistence_batch(clouds, sizes, dim, o, threads);   // warm-up: kernels, graph capture, buffers
    std::vector<double> run_s;
    gb300::BatchTiming tm, sum;
    for (int r = 0; r < reps; ++r) {
        const auto t0 = clk::now();
        res = gb300::persistence_batch(clouds, sizes, dim, o, threads, &tm);
        run_s.push_back(std::chrono::duration<double>(clk::now() - t0).count());
        sum.front_s += tm.front_s / reps;
        sum.copy_s += tm.copy_s / reps;
        sum.reduce_s += tm.reduce_s / reps;
    }
    // the same batch with the engine's own leftover-coface scan (no device
    // predicate): the diagrams must not change, only the host time
    gb300::BatchTiming tn;
    const auto res_np = gb300::persistence_batch(clouds, sizes, dim, o, threads, &tn, false);
    bool same_np = res_np.size() == res.size();
    for (size_t q = 0; same_np && q < res.size(); ++q)
        for (u32 d = 0; d <= o.maxdim && same_np; ++d)
            same_np = res[q].barcode.birth[d] == res_np[q].barcode.birth[d] &&
                      res[q].barcode.death[d] == res_np[q].barcode.death[d];
    u64 bars = 0;
    for (const Result& r : res)
        for (u32 d = 0; d < r.barcode.ndims(); ++d) bars += r.barcode.birth[d].size();
    // the reference, cloud by cloud, on every stride-th cloud
    double ref_s = 0;
    u32 compared = 0;
    bool same = true;
    if (stride)
        for (u32 q = 0; q < count; q += stride) {
            const auto t0 = clk::now();
            const Result ref = persistence(clouds[q], sizes[q], dim, o);
            ref_s += std::chrono::duration<double>(clk::now() - t0).count();
            for (u32 d = 0; d <= o.maxdim; ++d) same = same && canon(ref.barcode, d) == canon(res[q].barcode, d);
            ++compared;
        }
    double mean = 0;
    for (double s : run_s) mean += s / run_s.size();
    std::printf("{\"clouds\": %u, \"points\": %llu, \"bars\": %llu, \"batch_s\": %.6f, \"front_s\": %.6f, "
                "\"copy_s\": %.6f, \"reduce_s\": %.6f, \"threads\": %u, \"reps\": %d, \"reference_s\": %.6f, "
                "\"reference_clouds\": %u, \"identical\": %s, \"reduce_s_without_device_predicate\": %.6f, "
                "\"same_without_device_predicate\": %s}\n",
                count, (unsigned long long)total, (unsigned long long)bars, mean, sum.front_s, sum.copy_s,
                sum.reduce_s, threads ? threads : std::thread::hardware_concurrency(), reps, ref_s, compared,
                same ? "true" : "false", tn.reduce_s, same_np ? "true" : "false");
    return same && same_np ? 0 : 1;
}
