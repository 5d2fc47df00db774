// tt_redzed_pred.cu — RedZeD's static leftover-coface predicate on the device.
//
// The reference's RedZeD engine (redzed.hpp:1261-1273) asks, for every edge e
// = (u, v), u < v, that closes a cycle at maxdim 1, whether a triangle on e
// that step 1 of its active enumeration did not reach already exists:
// has_leftover_coface (:1238-1241) -> DenseGeom::any_common_radius_neighbor
// (:728-765) with coface_ready (:1193-1202). When step 1 found no candidate
// vertex (nothing is excluded; the engine calls it so on most edges), the
// answer depends only on the distances:
//   some w other than u and v with d(u, w) <= d(e) and d(v, w) <= d(e) (the
//   radius graph of the edges up to d(e), which advance_radius has grown to)
//   for which x u {w} is ready: w < u always; u < w < v when d(w, v) < d(e);
//   w > v when d(w, u) < d(e) and d(w, v) < d(e) (the younger faces must be
//   strictly shorter, as coface_ready's position masks require for an edge).
// k_leftover computes it for every kept pair at once, one warp a pair over
// coalesced row chunks, starting at u's chunk and stopping at the first
// witness. The host engine reads the answer instead of scanning the radius
// graph whenever no vertex is excluded, and runs its own scan otherwise, so
// the diagram cannot change.
#include "tt_internal.cuh"

namespace tt {

namespace {

__global__ void k_leftover(const f32* __restrict__ mat, u32 n, f32 thr, u32 words, u64 pairs,
                           unsigned long long* __restrict__ bits) {
    const u32 lane = threadIdx.x & 31;
    const u64 warps = (u64(gridDim.x) * blockDim.x) >> 5;
    const u32 chunks = (n + 31) / 32;
    for (u64 t = (u64(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; t < pairs; t += warps) {
        u32 v, u;
        decode_edge(t, v, u);   // v > u
        const f32 d = mat[u64(u) * n + v];
        if (!(d <= thr)) continue;
        const f32* ru = mat + u64(u) * n;
        const f32* rv = mat + u64(v) * n;
        bool found = false;
        for (u32 q = 0; q < chunks && !found; ++q) {
            u32 ch = (u >> 5) + q;
            if (ch >= chunks) ch -= chunks;
            const u32 w = ch * 32 + lane;
            bool ok = false;
            if (w < n && w != u && w != v) {
                const f32 du = ru[w], dv = rv[w];
                const bool adj = du <= d && dv <= d;
                const bool ready = w < u || (w < v ? dv < d : (du < d && dv < d));
                ok = adj && ready;
            }
            found = __any_sync(0xffffffffu, ok);
        }
        if (lane == 0 && found) atomicOr(&bits[u64(u) * words + (v >> 6)], 1ull << (v & 63));
    }
}

}  // namespace

// bits (device, n x ceil(n / 64) words): bit (u, v), u < v, set when the
// kept edge (u, v) has a leftover coface with nothing excluded.
void redzed_leftover(tt_ctx* c, const f32* mat, u32 n, f32 thr, unsigned long long* bits) {
    const u32 words = (n + 63) / 64;
    TT_CUDA(cudaMemsetAsync(bits, 0, sizeof(u64) * u64(n) * words, c->stream));
    const u64 pairs = u64(n) * (n > 0 ? n - 1 : 0) / 2;
    if (!pairs) return;
    const u32 grid = u32(std::min<u64>((pairs * 32 + 255) / 256, u64(c->sms) * 32));
    k_leftover<<<grid, 256, 0, c->stream>>>(mat, n, thr, words, pairs, bits);
    TT_LAUNCH("k_leftover");
    ++c->launches;
}

}  // namespace tt
