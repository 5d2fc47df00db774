// tt_knn_tc.cu — exact L2 k nearest neighbours in R^32 with a tensor-core
// (tcgen05) Gram filter and a bounding-ball tile order.
//
// Same result as the exhaustive scan (tt_scan.cuh KnnOp, which replaces
// graph.hpp knn_lists_exact :211-225): the k smallest (distance, id) pairs
// per query, every distance the reference's lane-ordered float32 l2
// (metric.hpp:92-112), ties broken by the smaller original id. Two exact
// tests decide which candidates are worth that evaluation; neither can
// change a list.
//
// 1. Tiles. The points are regrouped (a stable sort by nearest pivot, the
//    pivots strided samples chained nearest-first) so that a 128-point tile
//    is compact; every tile keeps its centroid c and radius R = max |x - c|.
//    A query q with current k-th distance d_k skips a tile when
//    |q - c| > d_k + R (with margins for every rounding, see the lookahead
//    product in the kernel): by the triangle inequality no point of the tile
//    can then enter the list. A query block visits the tiles outward from
//    its own (B, B+1, B-1, ...), tests them in batches (one tensor-core
//    product of the queries with up to 128 centroids each), and loads only
//    the tiles some query of the block still needs; a warp skips a loaded
//    tile that none of its queries needs.
// 2. Gram filter. The regrouped copy keeps every coordinate as a TF32-exact
//    head x~ (13 low mantissa bits cleared) plus those bits in a side array,
//    so the tensor core multiplies exact values and the exact path
//    reassembles x bit for bit. For a loaded tile the tensor core produces
//      D(q, c) = q~ . c~ - W(c),   W(c) <= |c~|^2 (1 - 2^-16) / 2,
//    the norm term entering as a fifth K-step (two TF32-exact parts). Only
//    the FP32 accumulation rounds, by at most E = 2^-17 S, S = |q~|^2 +
//    |c~|^2 (the accumulation bound below; k_tc_gram_check measures under
//    2^-22 S on GB300), so
//      L = |q~|^2 (1 - 2^-16) - 2 D <= |q~ - c~|^2,
//    and with e_x >= |x - x~| (per point, rounded up) the true distance is
//    at least sqrt(L) - e_q - e_c. A candidate is evaluated exactly when
//      L <= (sqrt(T_q) + e_q + e_T)^2,   T_q = sq_bound(d_k) (1 + 2^-16),
//    e_T the tile's largest e_c, so every candidate whose lane-ordered
//    distance could enter the list passes (the 2^-16 in T_q covers the
//    lane-ordered sum's own rounding). The margins are absolute (of the
//    order of the TF32 rounding of the points, times d_k), not relative to
//    |q|^2 + |c|^2: points far from the origin filter as tightly as points
//    near it. The epilogue is a max over the accumulator row and one
//    compare.
//
// The accumulation bound. The products of TF32-exact operands are exact
// (11-bit significands: 22 bits, within FP32's 24), and every product and
// every partial sum of the exact values is at most |q~| |c~| <= S / 2 in
// magnitude. The filter assumes one thing of the tensor core's FP32
// accumulation: each accumulation step adds a block of b products (b in
// {1, 2, 4, 8}) to the running sum by aligning the terms to the largest and
// keeping at least 24 significant bits of it (truncating or rounding the
// rest), then normalises the result to FP32 (within one unit in its last
// place). That is the behaviour the published studies of NVIDIA tensor
// cores measured (products exact, alignment to the largest term, truncation,
// 24 bits or more), and it is the weakest of them. A step then errs by less
// than 2^-24 S per aligned term (b products and the running sum) plus 2^-24 S
// for the normalisation: (b + 2) 2^-24 S a step, (8 / b) steps a K = 8
// instruction, at most 24 x 2^-24 S an instruction (b = 1), and the five
// instructions of a tile product (four over the coordinates, one over the
// norm term) at most 120 x 2^-24 S < E = 2^-17 S. Every margin below is
// derived for E; the lookahead product (four instructions) has the same
// bound with S = |q~|^2 + |c|^2.
//
// Pipeline per CTA (128 threads = 4 warps, one query row per thread, 128
// queries per block, persistent over query blocks):
//   TMA (cp.async.bulk.tensor, 128-byte swizzle) loads the query tile once
//   and the chosen candidate tiles into two shared-memory stages, each with
//   one bulk copy of the tile's pack (low bits, augmentation rows, ids,
//   record tail); warp 1 issues a stage's copies as soon as the stage is
//   free. The first warp to finish a tile's epilogue issues tcgen05.mma.kind::tf32
//   (M = 128, N = 128, 5 x K = 8) for the next tile into the free one of two
//   TMEM accumulators and commits to an mbarrier; the tensor core runs it
//   while the other warps finish the current tile, reading its Gram
//   rows (tcgen05.ld 32x32b.x32, two loads in flight), filtering and running
//   the exact path. One barrier a tile.
// TMEM: 2 x 128 columns per CTA; shared memory is padded so that at most two
// CTAs share an SM, so tcgen05.alloc never waits. Every mbarrier wait is
// bounded (tt_tma.cuh); on a timeout the kernel records the error, waits
// (bounded) for its copies and products in flight, and still frees its TMEM.
#include <cuda.h>

#include <algorithm>

#include "tt_internal.cuh"
#include "tt_metric.cuh"
#include "tt_tma.cuh"

namespace tt {

namespace {

constexpr int TC_DIM = 32;      // coordinates per point (one 128-byte swizzle row)
constexpr int TC_M = 128;       // queries per block (TMEM lanes)
constexpr int TC_N = 128;       // candidates per tile (accumulator columns)
constexpr int TC_K = 16;        // register top-k capacity
constexpr u32 TILE_BYTES = TC_M * TC_DIM * 4;   // 16 KiB (query and candidate tiles alike)
constexpr int TC_Q = 256;                       // survivor queue per warp (pairs)
constexpr int NSTAGE = 2;                       // candidate tiles in flight (TMA ring)
constexpr u32 TC_TEST = 128;                    // most positions tested per lookahead batch (one N = 128 product)
constexpr int ST_STRIDE = 36;                   // floats per tile record: centroid, R, |centroid|^2, largest e, largest nq
constexpr int MAX_PIV = 128;
constexpr size_t TC_SMEM = 110 * 1024;          // two CTAs per SM (2 x (110 + 1) KiB of 228)
static_assert(NSTAGE == 2, "the stage bookkeeping below assumes two stages");
static_assert(TC_M == TC_N, "query blocks and candidate tiles share one tiling");

constexpr u32 AUG_BYTES = TC_N * 16;  // augmentation rows per tile (one 16-byte core-matrix row each)
constexpr u32 ID_BYTES = TC_N * 4;    // original ids per tile
constexpr u32 LO_BYTES = TC_N * TC_DIM * 2;   // low mantissa bits per tile (u16 per coordinate)
// A tile's pack: everything but the TF32 heads, one bulk copy: the low bits,
// the augmentation rows, the original ids and the record tail (R, |c|^2,
// largest e, largest nq).
constexpr u32 PK_AUG = LO_BYTES;
constexpr u32 PK_ID = PK_AUG + AUG_BYTES;
constexpr u32 PK_TAIL = PK_ID + ID_BYTES;
constexpr u32 PACK_BYTES = PK_TAIL + 16;
static_assert(PACK_BYTES % 16 == 0, "bulk copies move multiples of 16 bytes");

// The fifth K-step of every product adds the candidate's norm term: the
// query side holds rows (1, 1, 0, 0 | 0, 0, 0, 0), the candidate side
// (w_hi, w_lo, 0, 0 | 0, 0, 0, 0) with -w_hi - w_lo <= |c~|^2 (1 - 2^-16) / 2
// (two TF32-exact parts), so the accumulator holds D = G + w_hi + w_lo and
// the filter is a compare against it.
// Layout: no swizzle, K-major, 8-row core matrices of 16-byte rows; the
// first K half of row r at r * 16 (so a tile's rows are one contiguous 2 KiB
// copy), the second K half in a shared 2 KiB block of zeros placed above
// both first halves (the descriptors' leading offsets are positive).
struct Shared {
    alignas(1024) float4 aaug[TC_M];         // (1, 1, 0, 0) per query row
    alignas(1024) unsigned char a[TILE_BYTES];
    alignas(1024) unsigned char b[NSTAGE][TILE_BYTES];
    alignas(16) u16 alo[TC_M * TC_DIM];  // the query tile's low mantissa bits
    alignas(16) unsigned char pk[NSTAGE][PACK_BYTES];   // the stage tiles' packs
    float4 zeros[TC_N];                  // the second K half of both augmentation sides
    u32 q[4][TC_Q];                      // per-warp survivor queue: owner lane << 7 | candidate row
    f32 r[4][TC_Q];                      // their exact distances
    u32 need[2][4][TC_TEST / 32];        // per-warp lookahead masks (double-buffered)
    alignas(1024) unsigned char cent[TC_TEST * 128];   // lookahead batch centroids, 128-byte swizzled (MMA operand)
    alignas(16) float2 trc[TC_TEST];     // their radius and |centroid|^2
    alignas(8) u64 bar_a;
    alignas(8) u64 bar_b[NSTAGE];
    alignas(8) u64 bar_mma[2];
    alignas(8) u64 bar_t;                // lookahead product done
    u32 tmem_base;
    u32 block;
    u32 stop[2];
    u32 ticket[2];                       // warps done with tile it's epilogue (by tile parity)
    volatile u32 fail;                   // a bounded wait of this CTA timed out
};

static_assert(sizeof(Shared) + 1024 <= TC_SMEM, "shared layout (plus alignment slack) exceeds the reservation");

// Row r (0..127) of a 128-byte-swizzled tile: 16-byte chunk c of the row sits
// at chunk position c ^ (r & 7) (the TMA / UMMA 128-byte swizzle).
__device__ __forceinline__ void swz_row(const unsigned char* tile, u32 r, f32 (&o)[TC_DIM]) {
#pragma unroll
    for (int ch = 0; ch < 8; ++ch) {
        const float4 t4 = *reinterpret_cast<const float4*>(tile + r * 128 + ((ch ^ (r & 7)) << 4));
        o[4 * ch] = t4.x;
        o[4 * ch + 1] = t4.y;
        o[4 * ch + 2] = t4.z;
        o[4 * ch + 3] = t4.w;
    }
}

// Row r of a tile reassembled: the TF32-exact head from the swizzled tile,
// the 13 low mantissa bits from the low-bits array (layout at k_tc_tiles).
__device__ __forceinline__ void raw_row(const unsigned char* tile, const u16* lo, u32 r, f32 (&o)[TC_DIM]) {
    swz_row(tile, r, o);
    const uint4* lr = reinterpret_cast<const uint4*>(lo + r * TC_DIM);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const uint4 t = lr[c ^ ((r >> 1) & 3u)];
        const u32 w[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
        for (int e = 0; e < 8; ++e)
            o[8 * c + e] = __uint_as_float(__float_as_uint(o[8 * c + e]) | ((w[e >> 1] >> (16 * (e & 1))) & 0xffffu));
    }
}

// UMMA shared-memory descriptor: K-major operand, 128-byte swizzle, rows of
// 128 bytes in 1024-byte groups of 8 (stride byte offset 1024), version 1.
__device__ __forceinline__ u64 sw128_desc(u32 saddr) {
    return u64((saddr >> 4) & 0x3fff) | (u64(1) << 16) | (u64(1024 >> 4) << 32) | (u64(1) << 46) |
           (u64(2) << 61);
}

// UMMA shared-memory descriptor without swizzle, K-major: core matrices of
// 8 rows x 16 bytes; lbo = byte offset between core matrices adjacent in K,
// sbo = between core matrices adjacent in M / N.
__device__ __forceinline__ u64 plain_desc(u32 saddr, u32 lbo, u32 sbo) {
    return u64((saddr >> 4) & 0x3fff) | (u64((lbo >> 4) & 0x3fff) << 16) | (u64((sbo >> 4) & 0x3fff) << 32) |
           (u64(1) << 46);
}

// Instruction descriptor, kind::tf32: D f32, A/B tf32, both K-major, N, M.
constexpr u32 kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | (u32(TC_N >> 3) << 17) | (u32(TC_M >> 4) << 24);

// The lookahead product: M = 128 queries x N = TC_TEST centroids (the same
// shape as a tile product).
static_assert(TC_TEST == TC_N, "the lookahead product fills one accumulator");

__device__ __forceinline__ void tma_tile(void* dst, const CUtensorMap* map, int row, u64* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(smem_addr(dst)),
        "l"(map), "r"(0), "r"(row), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void mma_step(u32 d_tmem, u64 da, u64 db, u32 acc, u32 idesc = kIdesc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(da), "l"(db), "r"(idesc), "r"(acc)
        : "memory");
}

// D = A B^T over the 32 coordinates (4 K-steps on the swizzled tiles) plus
// the augmentation step (a_aug, b_aug: starts of the first K halves; z: the
// zero block holding both second halves).
__device__ __forceinline__ void mma_tile(u32 d_tmem, u32 a_saddr, u32 b_saddr, u32 a_aug, u32 b_aug, u32 z) {
#pragma unroll
    for (int ks = 0; ks < TC_DIM / 8; ++ks)   // K = 8 tf32 = 32 bytes per step
        mma_step(d_tmem, sw128_desc(a_saddr + 32 * ks), sw128_desc(b_saddr + 32 * ks), ks > 0);
    mma_step(d_tmem, plain_desc(a_aug, z - a_aug, 128), plain_desc(b_aug, z - b_aug, 128), 1);
}

// Ascending bitonic sort of N values held in registers (all indices are
// compile-time constants once unrolled). NaN must not be present.
template <int N>
__device__ __forceinline__ void bitonic_sort(f32 (&a)[N]) {
#pragma unroll
    for (int size = 2; size <= N; size <<= 1) {
#pragma unroll
        for (int stride = size / 2; stride > 0; stride >>= 1) {
#pragma unroll
            for (int i = 0; i < N; ++i) {
                const int j = i ^ stride;
                if (j > i) {
                    const f32 lo = fminf(a[i], a[j]), hi = fmaxf(a[i], a[j]);
                    if ((i & size) == 0) {
                        a[i] = lo;
                        a[j] = hi;
                    } else {
                        a[i] = hi;
                        a[j] = lo;
                    }
                }
            }
        }
    }
}

// max of three (one instruction on sm_100 and later)
__device__ __forceinline__ f32 fmax3(f32 a, f32 b, f32 c) {
    f32 r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

__device__ __forceinline__ void mma_commit(u64* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld32(u32 taddr, u32 (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
          "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Two 32-column loads in flight at once: tmem_ld32_start issues one, and
// tmem_wait2 waits for both (every register tied to the wait, so that no
// use of a loaded value can be scheduled before it).
__device__ __forceinline__ void tmem_ld32_start(u32 taddr, u32 (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait2(u32 (&v)[32], u32 (&w)[32]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]), "+r"(v[6]), "+r"(v[7]), "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]), "+r"(v[12]), "+r"(v[13]), "+r"(v[14]), "+r"(v[15]), "+r"(v[16]), "+r"(v[17]), "+r"(v[18]), "+r"(v[19]), "+r"(v[20]), "+r"(v[21]), "+r"(v[22]), "+r"(v[23]), "+r"(v[24]), "+r"(v[25]), "+r"(v[26]), "+r"(v[27]), "+r"(v[28]), "+r"(v[29]), "+r"(v[30]), "+r"(v[31])
                 :
                 : "memory");
    asm volatile(""
                 : "+r"(w[0]), "+r"(w[1]), "+r"(w[2]), "+r"(w[3]), "+r"(w[4]), "+r"(w[5]), "+r"(w[6]), "+r"(w[7]), "+r"(w[8]), "+r"(w[9]), "+r"(w[10]), "+r"(w[11]), "+r"(w[12]), "+r"(w[13]), "+r"(w[14]), "+r"(w[15]), "+r"(w[16]), "+r"(w[17]), "+r"(w[18]), "+r"(w[19]), "+r"(w[20]), "+r"(w[21]), "+r"(w[22]), "+r"(w[23]), "+r"(w[24]), "+r"(w[25]), "+r"(w[26]), "+r"(w[27]), "+r"(w[28]), "+r"(w[29]), "+r"(w[30]), "+r"(w[31]));
}

__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }


template <int DIM>
struct RegVec {
    const f32 (&q)[DIM];
    __device__ __forceinline__ f32 operator()(u32 k) const { return q[k]; }
};

// Tile visited at step s by query block B: B, B+1, B-1, B+2, B-2, ... and,
// once one side is exhausted, the rest of the other side in order.
__device__ __forceinline__ u32 spiral_tile(u32 B, u32 s, u32 ntiles) {
    const u32 left = B, right = ntiles - 1 - B;
    const u32 m = min(left, right);
    if (s <= 2 * m) return s == 0 ? B : (s & 1) ? B + (s + 1) / 2 : B - s / 2;
    const u32 u = s - 2 * m;
    return right > left ? B + m + u : B - m - u;
}

// ---- tile order ------------------------------------------------------------

// Pivots: rows floor(p n / P) of x; rank[p] = position of pivot p on a
// nearest-first chain from pivot 0 (ties to the lower index), so that
// pivots of one region of space sit next to each other in the order.
// The block fills the P x P distance matrix in shared memory; one warp then
// walks the chain (two warp reductions per step: the smallest distance,
// then the lowest pivot index holding it; non-negative float bits order
// like the floats).
constexpr int PIV_THREADS = 1024;
__global__ void __launch_bounds__(PIV_THREADS) k_tc_pivots(const f32* __restrict__ x, u32 n, u32 P,
                                                          f32* __restrict__ piv, u32* __restrict__ rank) {
    pdl_wait();
    pdl_trigger();
    extern __shared__ f32 psm[];
    f32* pv = psm;                       // P x (TC_DIM + 1)
    f32* dm = psm + P * (TC_DIM + 1);    // P x P
    for (u32 t = threadIdx.x; t < P * TC_DIM; t += blockDim.x) {
        const u32 p = t / TC_DIM, k = t % TC_DIM;
        const f32 v = __ldg(x + (u64(p) * n / P) * TC_DIM + k);
        pv[p * (TC_DIM + 1) + k] = v;
        piv[u64(p) * TC_DIM + k] = v;
    }
    __syncthreads();
    for (u32 t = threadIdx.x; t < P * P; t += blockDim.x) {
        const u32 p = t / P, r = t % P;
        f32 d = 0.0f;
#pragma unroll 8
        for (int k = 0; k < TC_DIM; ++k) {
            const f32 u = pv[p * (TC_DIM + 1) + k] - pv[r * (TC_DIM + 1) + k];
            d = fmaf(u, u, d);
        }
        dm[t] = d;
    }
    __syncthreads();
    if (threadIdx.x >= 32) return;
    const u32 lane = threadIdx.x;
    u32 visited = lane == 0 ? 1u : 0u;   // bit i: pivot lane + 32 i is on the chain
    if (lane == 0) rank[0] = 0;
    u32 cur = 0;
    for (u32 step = 1; step < P; ++step) {
        u32 bd = 0xffffffffu, bp = 0xffffffffu;   // this lane's nearest unvisited pivot
        for (u32 i = 0, p = lane; p < P; ++i, p += 32) {
            const u32 db = fbits(dm[cur * P + p]);
            if (!((visited >> i) & 1u) && (bp == 0xffffffffu || db < bd)) {
                bd = db;
                bp = p;
            }
        }
        const u32 md = __reduce_min_sync(0xffffffffu, bd);
        cur = __reduce_min_sync(0xffffffffu, bp != 0xffffffffu && bd == md ? bp : 0xffffffffu);
        if (lane == 0) rank[cur] = step;
        if ((cur & 31u) == lane) visited |= 1u << (cur >> 5);
    }
}

// key[i] = the nearest pivot of point i (ties to the lower pivot index; the
// pivots are rows floor(p n / P), read from x, so this runs beside the chain
// of k_tc_pivots and k_tc_rank maps the index to the chain's rank), val[i] =
// i. Two points a thread; the distance order comes
// from |p|^2 - 2 x.p (the assignment only shapes the tile order: any
// nearest-pivot choice leaves the lists unchanged).
__global__ void k_tc_assign(const f32* __restrict__ x, u32 n, u32 P, u64* __restrict__ key, u32* __restrict__ val) {
    pdl_wait();
    pdl_trigger();
    extern __shared__ float4 sp4[];      // P x 8 float4 (the pivots: rows floor(p n / P)), then P norms
    f32* pn = reinterpret_cast<f32*>(sp4 + P * 8);
    for (u32 t = threadIdx.x; t < P * 8; t += blockDim.x)
        sp4[t] = __ldg(reinterpret_cast<const float4*>(x + (u64(t / 8) * n / P) * TC_DIM) + t % 8);
    __syncthreads();
    for (u32 p = threadIdx.x; p < P; p += blockDim.x) {
        f32 s = 0.0f;
#pragma unroll
        for (int ch = 0; ch < 8; ++ch) {
            const float4 c = sp4[p * 8 + ch];
            s = fmaf(c.x, c.x, fmaf(c.y, c.y, fmaf(c.z, c.z, fmaf(c.w, c.w, s))));
        }
        pn[p] = s;
    }
    __syncthreads();
    const u32 i0 = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    if (i0 >= n) return;
    const u32 i1 = min(i0 + 1, n - 1);
    f32 q0[TC_DIM], q1[TC_DIM];
#pragma unroll
    for (int ch = 0; ch < 8; ++ch) {
        const float4 a = __ldg(reinterpret_cast<const float4*>(x + u64(i0) * TC_DIM) + ch);
        const float4 b = __ldg(reinterpret_cast<const float4*>(x + u64(i1) * TC_DIM) + ch);
        q0[4 * ch] = a.x, q0[4 * ch + 1] = a.y, q0[4 * ch + 2] = a.z, q0[4 * ch + 3] = a.w;
        q1[4 * ch] = b.x, q1[4 * ch + 1] = b.y, q1[4 * ch + 2] = b.z, q1[4 * ch + 3] = b.w;
    }
    u32 b0 = 0, b1 = 0;
    f32 d0 = INFINITY, d1 = INFINITY;
    for (u32 p = 0; p < P; ++p) {
        f32 s0 = 0.0f, s1 = 0.0f;
#pragma unroll
        for (int ch = 0; ch < 8; ++ch) {
            const float4 c = sp4[p * 8 + ch];
            s0 = fmaf(q0[4 * ch], c.x, fmaf(q0[4 * ch + 1], c.y, fmaf(q0[4 * ch + 2], c.z, fmaf(q0[4 * ch + 3], c.w, s0))));
            s1 = fmaf(q1[4 * ch], c.x, fmaf(q1[4 * ch + 1], c.y, fmaf(q1[4 * ch + 2], c.z, fmaf(q1[4 * ch + 3], c.w, s1))));
        }
        const f32 e0 = fmaf(-2.0f, s0, pn[p]), e1 = fmaf(-2.0f, s1, pn[p]);
        if (e0 < d0) d0 = e0, b0 = p;
        if (e1 < d1) d1 = e1, b1 = p;
    }
    key[i0] = b0;
    val[i0] = i0;
    if (i0 + 1 < n) {
        key[i0 + 1] = b1;
        val[i0 + 1] = i0 + 1;
    }
}

// key[i] = chain rank of point i's nearest pivot (k_tc_assign leaves the
// pivot's index: the chain runs beside it, on the side stream).
__global__ void k_tc_rank(const u32* __restrict__ rank, u32 n, u64* __restrict__ key) {
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) key[i] = rank[u32(key[i])];
}

// First position of each cell (chain rank) in the rank-sorted keys; cell P
// ends the array.
__global__ void k_tc_cells(const u64* __restrict__ skey, u32 n, u32 P, u32* __restrict__ cell_off) {
    pdl_wait();
    pdl_trigger();
    for (u32 p = blockIdx.x * blockDim.x + threadIdx.x; p <= P; p += gridDim.x * blockDim.x) {
        u32 lo = 0, hi = n;
        while (lo < hi) {
            const u32 mid = (lo + hi) >> 1;
            if (skey[mid] < p) lo = mid + 1;
            else hi = mid;
        }
        cell_off[p] = lo;
    }
}

// Second level: every point of a cell (s points) joins the nearest of
// min(16, max(1, s / 128)) sub-pivots (the cell's points at strided
// positions, ties to the lower one); key = cell << 4 | sub-pivot, so that
// the tiles of a cell follow its sub-cells. k_tc_subpiv gathers the
// sub-pivots into a table (row cell * 16 + j, then |.|^2), one warp a row.
__host__ __device__ __forceinline__ u32 sub_count(u32 s) { return s / 128u < 1u ? 1u : s / 128u > 16u ? 16u : s / 128u; }

__global__ void k_tc_subpiv(const f32* __restrict__ x, const u32* __restrict__ perm, const u32* __restrict__ cell_off,
                            u32 P, f32* __restrict__ spv, f32* __restrict__ spn) {
    pdl_wait();
    pdl_trigger();
    const u32 wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (wid >= P * 16) return;
    const u32 cell = wid >> 4, j = wid & 15u;
    const u32 o = cell_off[cell], s = cell_off[cell + 1] - o;
    if (s == 0 || j >= sub_count(s)) return;
    const f32 v = __ldg(x + u64(perm[o + u32(u64(j) * s / sub_count(s))]) * TC_DIM + lane);
    spv[u64(wid) * TC_DIM + lane] = v;
    f32 q = v * v;
#pragma unroll
    for (int off = 16; off; off >>= 1) q += __shfl_xor_sync(0xffffffffu, q, off);
    if (lane == 0) spn[wid] = q;
}

__global__ void k_tc_assign2(const f32* __restrict__ x, u32 n, const u64* __restrict__ skey,
                             const u32* __restrict__ perm, const u32* __restrict__ cell_off,
                             const f32* __restrict__ spv, const f32* __restrict__ spn, u64* __restrict__ key2,
                             u32* __restrict__ val2) {
    pdl_wait();
    pdl_trigger();
    const u32 r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const u32 cell = u32(skey[r]);
    const u32 S = sub_count(cell_off[cell + 1] - cell_off[cell]);
    const u32 self = perm[r];
    f32 q[TC_DIM];
    const float4* xr = reinterpret_cast<const float4*>(x + u64(self) * TC_DIM);
#pragma unroll
    for (int ch = 0; ch < 8; ++ch) {
        const float4 t4 = __ldg(xr + ch);
        q[4 * ch] = t4.x;
        q[4 * ch + 1] = t4.y;
        q[4 * ch + 2] = t4.z;
        q[4 * ch + 3] = t4.w;
    }
    u32 best = 0;
    f32 bd = INFINITY;
    for (u32 j = 0; j < S; ++j) {
        const float4* pr = reinterpret_cast<const float4*>(spv + u64(cell * 16 + j) * TC_DIM);
        f32 d = 0.0f;
#pragma unroll
        for (int ch = 0; ch < 8; ++ch) {
            const float4 c = __ldg(pr + ch);
            d = fmaf(q[4 * ch], c.x, fmaf(q[4 * ch + 1], c.y, fmaf(q[4 * ch + 2], c.z, fmaf(q[4 * ch + 3], c.w, d))));
        }
        const f32 e = fmaf(-2.0f, d, __ldg(spn + cell * 16 + j));
        if (e < bd) {
            bd = e;
            best = j;
        }
    }
    key2[r] = (u64(cell) << 4) | best;
    val2[r] = self;
}

// The low-bits array: u16 per coordinate, 64 bytes per row, 16-byte chunk
// c (coordinates 8c..8c+7) of row r stored at chunk position c ^ ((r >> 1)
// & 3), so that eight consecutive rows read by one quarter-warp hit
// distinct banks.
// Regrouped copy in two parts, one block (128 threads) per tile, thread r
// on row T * 128 + r. xh[row]: the coordinates of x[perm[row]] with their
// 13 low mantissa bits cleared (TF32-exact: the tensor core multiplies them
// without rounding). lo[row]: those 13 bits, u16 per coordinate, so that
// xh | lo is the point again, bit for bit (the exact path's input). Per row:
// nq = |xh|^2 rounded down; e >= |x - xh| (rounded up; a coordinate below
// 2^-126 counts in full, in case the tensor core flushes it); the
// augmentation row (w_hi, w_lo, 0, 0) with
// -w_hi - w_lo in [W (1 - 2^-20), W], W = nq (1 - 2^-16) / 2 (two TF32-exact
// parts, both truncated toward zero); the original id. Rows [n, wpad) are
// padding (augmentation -3e38: never passes; id ~0). Then the tile record:
// centroid (the mean of the rows, rounded to TF32 so that it enters the
// lookahead product exactly; the bound holds for every centre), radius
// sqrt(max |x - c|^2) (a NaN coordinate makes it NaN: the tile is then never
// skipped), |c|^2, and the tile's largest e and nq (the Gram filter's
// per-tile error terms).
__global__ void __launch_bounds__(TC_N) k_tc_tiles(const f32* __restrict__ x, u32 n, const u32* __restrict__ perm,
                                                  f32* __restrict__ xh, unsigned char* __restrict__ pack,
                                                  f32* __restrict__ nq, f32* __restrict__ eq, f32* __restrict__ stats) {
    pdl_wait();
    pdl_trigger();
    __shared__ f32 rows[TC_N][TC_DIM + 1];
    __shared__ f32 part[4][TC_DIM];
    __shared__ f32 cent[TC_DIM];
    __shared__ f32 red[3][4];
    const u32 T = blockIdx.x, t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const u32 r = T * TC_N + t;
    const bool live = r < n;
    f32 v[TC_DIM];
    f32 s = 0.0f, e2 = 0.0f;
    unsigned char* pt = pack + u64(T) * PACK_BYTES;
    uint4* lr = reinterpret_cast<uint4*>(pt) + 4 * t;
    float4* aug = reinterpret_cast<float4*>(pt + PK_AUG);
    u32* ids = reinterpret_cast<u32*>(pt + PK_ID);
    if (live) {
        const u32 src = perm[r];
        const float4* xr = reinterpret_cast<const float4*>(x + u64(src) * TC_DIM);
        float4* xo = reinterpret_cast<float4*>(xh + u64(r) * TC_DIM);
        u32 lw[16];   // the low bits, two coordinates per word
#pragma unroll
        for (int ch = 0; ch < 8; ++ch) {
            const float4 t4 = __ldg(xr + ch);
            v[4 * ch] = t4.x, v[4 * ch + 1] = t4.y, v[4 * ch + 2] = t4.z, v[4 * ch + 3] = t4.w;
            f32 h[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const f32 ve = v[4 * ch + e];
                const u32 u = __float_as_uint(ve);
                h[e] = __uint_as_float(u & 0xffffe000u);
                s = __fmaf_rd(h[e], h[e], s);   // exact products (11-bit significands), sum rounded down
                const f32 b = fabsf(ve) < 0x1p-126f ? fabsf(ve) : fabsf(ve - h[e]);
                e2 = __fmaf_ru(b, b, e2);
                const u32 l = u & 0x1fffu;
                if (e & 1) lw[2 * ch + (e >> 1)] |= l << 16;
                else lw[2 * ch + (e >> 1)] = l;
            }
            xo[ch] = make_float4(h[0], h[1], h[2], h[3]);
        }
#pragma unroll
        for (int c = 0; c < 4; ++c)
            lr[c ^ ((r >> 1) & 3u)] = make_uint4(lw[4 * c], lw[4 * c + 1], lw[4 * c + 2], lw[4 * c + 3]);
        const f32 w = -__fmul_rd(s, 0.5f * (1.0f - 0x1p-16f));
        // head and remainder, both truncated toward zero; a non-finite w keeps
        // its head and gets a zero tail
        const f32 hi = __uint_as_float(__float_as_uint(w) & 0xffffe000u);
        const f32 rem = isfinite(w) ? w - hi : 0.0f;   // exact
        aug[t] = make_float4(hi, __uint_as_float(__float_as_uint(rem) & 0xffffe000u), 0.0f, 0.0f);
        ids[t] = src;
        e2 = __fsqrt_ru(e2);
    } else {
#pragma unroll
        for (int k = 0; k < TC_DIM; ++k) v[k] = 0.0f;
        aug[t] = make_float4(-3.0e38f, 0.0f, 0.0f, 0.0f);
        ids[t] = 0xffffffffu;
#pragma unroll
        for (int c = 0; c < 4; ++c) lr[c] = make_uint4(0u, 0u, 0u, 0u);
    }
    nq[r] = s;
    eq[r] = e2;
    // centroid: column sums through shared memory (rows of 33 floats: no bank conflicts)
#pragma unroll
    for (int k = 0; k < TC_DIM; ++k) rows[t][k] = v[k];
    __syncthreads();
    {
        f32 cs = 0.0f;
        for (u32 q = warp * 32; q < warp * 32 + 32; ++q) cs += rows[q][lane];
        part[warp][lane] = cs;
    }
    __syncthreads();
    const u32 cnt = min(u32(TC_N), n - T * TC_N);
    if (t < 32) {
        const f32 sum = (part[0][t] + part[1][t]) + (part[2][t] + part[3][t]);
        const f32 c = __uint_as_float(__float_as_uint(sum / f32(cnt)) & 0xffffe000u);
        cent[t] = c;
        f32 cc = c * c;
#pragma unroll
        for (int o = 16; o; o >>= 1) cc += __shfl_xor_sync(0xffffffffu, cc, o);
        if (t == 0) stats[u64(T) * ST_STRIDE + 33] = cc;
        stats[u64(T) * ST_STRIDE + t] = c;
    }
    __syncthreads();
    f32 d = 0.0f;
    if (live) {
#pragma unroll
        for (int k = 0; k < TC_DIM; ++k) {
            const f32 u = v[k] - cent[k];
            d = fmaf(u, u, d);
        }
    }
    f32 em = e2, nm = s;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const f32 od = __shfl_xor_sync(0xffffffffu, d, o);
        d = (d != d || od != od) ? d + od : fmaxf(d, od);   // NaN is sticky
        em = fmaxf(em, __shfl_xor_sync(0xffffffffu, em, o));
        nm = fmaxf(nm, __shfl_xor_sync(0xffffffffu, nm, o));
    }
    if (lane == 0) {
        red[0][warp] = d;
        red[1][warp] = em;
        red[2][warp] = nm;
    }
    __syncthreads();
    if (t == 0) {
        f32 r2 = red[0][0], e = red[1][0], nmax = red[2][0];
        for (int q = 1; q < 4; ++q) {
            r2 = (r2 != r2 || red[0][q] != red[0][q]) ? r2 + red[0][q] : fmaxf(r2, red[0][q]);
            e = fmaxf(e, red[1][q]);
            nmax = fmaxf(nmax, red[2][q]);
        }
        f32* o = stats + u64(T) * ST_STRIDE;
        o[32] = sqrtf(r2);
        o[34] = e;
        o[35] = nmax;
        reinterpret_cast<float4*>(pt + PK_TAIL)[0] = make_float4(o[32], o[33], e, nmax);
    }
}

// ---- the kNN kernel ---------------------------------------------------------

__global__ void __launch_bounds__(128, 2)
k_knn_tc(const __grid_constant__ CUtensorMap map, const unsigned char* __restrict__ pack, const f32* __restrict__ eq,
         u32 n, u32 k, const f32* __restrict__ nq,
         const f32* __restrict__ stats, u32* __restrict__ ids, f32* __restrict__ dists, u32* __restrict__ next_block,
         u32* __restrict__ err, unsigned long long* __restrict__ counters) {
    pdl_wait();
    pdl_trigger();
    extern __shared__ unsigned char smem_raw[];
    Shared& S = *reinterpret_cast<Shared*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const u32 tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const u32 nblocks = (n + TC_M - 1) / TC_M;
    const u32 ntiles = nblocks;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&S.tmem_base)),
                     "r"(2 * TC_N)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    S.aaug[tid] = make_float4(1.0f, 1.0f, 0.0f, 0.0f);
    S.zeros[tid] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // visible to the tensor core
    if (tid == 0) {
        mbar_init(&S.bar_a, 1);
        for (int q = 0; q < NSTAGE; ++q) mbar_init(&S.bar_b[q], 1);
        mbar_init(&S.bar_mma[0], 1);
        mbar_init(&S.bar_mma[1], 1);
        mbar_init(&S.bar_t, 1);
        fence_mbar_init();
        S.stop[0] = S.stop[1] = 0;
        S.ticket[0] = S.ticket[1] = 0;
        S.fail = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const u32 tmem = S.tmem_base;
    u32 ph_a = 0, ub0 = 0, ub1 = 0, um0 = 0, um1 = 0;   // completed phases per stage / accumulator
    u32 ut = 0;                                          // completed lookahead products
    unsigned long long exact_evals = 0, tiles_done = 0;
    u32 npar = 0;   // S.need buffer of the next lookahead
    bool failed = false;

    // stage s <- candidate tile T: the TF32 heads (TMA, swizzled) and the pack
    auto load_stage = [&](int s, u32 T) {
        mbar_expect_tx(&S.bar_b[s], TILE_BYTES + PACK_BYTES);
        tma_tile(S.b[s], &map, int(T * TC_N), &S.bar_b[s]);
        bulk_g2s(S.pk[s], pack + u64(T) * PACK_BYTES, PACK_BYTES, &S.bar_b[s]);
    };

    for (;;) {
        if (tid == 0) S.block = atomicAdd(next_block, 1u);
        __syncthreads();
        const u32 blk = S.block;
        if (blk >= nblocks || failed) break;
        const u32 q0 = blk * TC_M;
        if (tid == 0) {
            // the previous block's generic reads of the query tile (survivor
            // queue) are ordered before this async-proxy overwrite
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_expect_tx(&S.bar_a, TILE_BYTES + LO_BYTES);
            tma_tile(S.a, &map, int(q0), &S.bar_a);
            bulk_g2s(S.alo, pack + u64(blk) * PACK_BYTES, LO_BYTES, &S.bar_a);
        }
        const u32 row = warp * 32 + lane;
        const u32 i = q0 + row;   // regrouped index of this thread's query
        const bool active = i < n;
        const f32 nqi = active ? nq[i] : 0.0f;            // |q~|^2 (rounded down), q~ the TF32 head
        const f32 eqi = active ? eq[i] : 0.0f;            // >= |q - q~|
        const f32 nql = __fmul_rd(nqi, 1.0f - 0x1p-16f);
        // Sorted list of keys (distance bits << 32 | original id): distances
        // are >= +0, so unsigned key order is the (distance, id) order of the
        // lists, ties to the smaller id. Its first TC_K - k slots hold the
        // sentinel 0 (no key is below it and none moves past it), so the
        // k-th entry is always lk[TC_K - 1] (every index a compile-time
        // constant: the list stays in registers); empty slots hold (+inf, ~0).
        u64 lk[TC_K];
#pragma unroll
        for (int t = 0; t < TC_K; ++t) lk[t] = u32(t) < TC_K - k ? 0ull : 0x7f800000ffffffffull;
        f32 sq = INFINITY;   // >= the true distance of any candidate that can still enter, plus |q - q~|
        f32 dk = INFINITY;   // current k-th distance
        // insert (d, j) into the sorted top-TC_K list; true if it entered.
        // c_s = (lk[s - 1] > key) is monotone in s, so slot s takes lk[s - 1]
        // where c_s holds, the key where c_s fails but c_{s + 1} holds, and
        // keeps its entry otherwise: independent compares and selects (a
        // NaN distance orders above +inf and never enters).
        auto consider = [&](u32 j, f32 d) -> bool {
            ++exact_evals;
            const u64 key = (u64(__float_as_uint(d)) << 32) | j;
            if (!(key < lk[TC_K - 1])) return false;
            bool above = true;   // c_{s + 1}
#pragma unroll
            for (int s = TC_K - 1; s >= 1; --s) {
                const bool c = lk[s - 1] > key;
                lk[s] = c ? lk[s - 1] : above ? key : lk[s];
                above = c;
            }
            if (above) lk[0] = key;
            return true;
        };
        // filter bound from the k-th entry; +inf until the list holds k. A
        // candidate whose lane-ordered distance can tie or beat d has true
        // squared distance <= sq_bound(d) (1 + 2^-16) (the sum's own rounding).
        auto update_bound = [&]() {
            const f32 d = __uint_as_float(u32(lk[TC_K - 1] >> 32));
            dk = d;
            // the filter's relative error bounds need |q|^2 far above the
            // subnormal range: below 2^-60 every candidate is evaluated
            sq = d < INFINITY && nqi >= 0x1p-60f ? __fadd_ru(__fsqrt_ru(__fmul_ru(sq_bound(d), 1.0f + 0x1p-16f)), eqi)
                                                 : INFINITY;
        };
        // Lookahead over the outward order (block-uniform state): bm holds the
        // positions of the current batch that some query of the block needs,
        // my the ones this thread's query needs (bit b of word c: position
        // bbase + 32 c + b).
        u32 sp = 0, bbase = 0;
        u32 bm0 = 0, bm1 = 0, bm2 = 0, bm3 = 0, my0 = 0, my1 = 0, my2 = 0, my3 = 0;
        static_assert(TC_TEST == 128, "four mask words");
        // acc: TMEM address of an accumulator the tile loop does not use right
        // now (the lookahead product fills it), or ~0u before the first tile
        // (every k-th distance is still +inf then). Batches grow with the
        // distance from the block's own tile (2, 8, 10, 20, 40, ..., 128
        // positions) so that the first ones are tested with fresh distances.
        auto refill = [&](u32 acc) {
            const u32 w = sp == 0 ? u32(NSTAGE) : min(TC_TEST, max(8u, sp));
            u32 m0 = 0, m1 = 0, m2 = 0, m3 = 0;
            if (acc == ~0u) {
                if (active)
                    m0 = (w >= 32 ? ~0u : (1u << w) - 1u) & (ntiles - sp >= 32 ? ~0u : (1u << (ntiles - sp)) - 1u);
            } else {
                {   // the batch's records: centroid (MMA operand, row = position); R (1 + 2^-16)
                    // and |centroid|^2 (1 - 2^-16) - 2^-120, each rounded outward
                    const u32 pos = sp + tid;
                    if (tid < w && pos < ntiles) {
                        const float4* rec =
                            reinterpret_cast<const float4*>(stats + u64(spiral_tile(blk, pos, ntiles)) * ST_STRIDE);
#pragma unroll
                        for (int ch = 0; ch < 8; ++ch)
                            *reinterpret_cast<float4*>(S.cent + tid * 128 + ((ch ^ (tid & 7)) << 4)) = __ldg(rec + ch);
                        const float4 rc = __ldg(rec + 8);
                        S.trc[tid] = make_float2(__fmul_ru(rc.x, 1.0f + 0x1p-16f),
                                                 __fsub_rd(__fmul_rd(rc.y, 1.0f - 0x1p-16f), 0x1p-120f));
                    }
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // centroids -> tensor core
                __syncthreads();
                // G = q~ . c for the 128 queries x the batch's centroids on the
                // tensor core. Both operands are TF32-exact (q~: the query's
                // head; c: rounded when the record was made), so the products
                // are exact and only the FP32 accumulation rounds:
                // |G - q~.c| <= 2^-17 (|q~|^2 + |c|^2) (the accumulation
                // bound). With s2 = nq + |c|^2 (nq rounded down, |c|^2 within
                // 2^-19),
                //   lower = s2 (1 - 2^-16) - 2 G - 2^-120 <= |q~ - c|^2
                // (rounded down; the absolute term covers products in the
                // subnormal range),
                // and |q - c| >= |q~ - c| - e_q. A tile is skipped when
                // lower > (sq + R (1 + 2^-16))^2, sq = sqrt(T) + e_q (T the
                // squared-distance bound of an entering candidate, rounded
                // up): then every point x of the tile has |q - x| >=
                // |q - c| - R > sqrt(T) (R is within 2^-18 of the tile's
                // largest distance to c), so it can neither beat nor tie the
                // k-th entry. dk below 2^-50, |q|^2 below 2^-60 (where
                // underflow defeats relative bounds), any non-finite value
                // and any NaN keep the tile.
                if (tid == 0) {
                    tc_fence_after();
#pragma unroll
                    for (int ks = 0; ks < TC_DIM / 8; ++ks)
                        mma_step(acc, sw128_desc(smem_addr(S.a) + 32 * ks), sw128_desc(smem_addr(S.cent) + 32 * ks),
                                 ks > 0);
                    mma_commit(&S.bar_t);
                }
                mbar_wait(&S.bar_t, ut & 1, err, &S.fail);
                ++ut;
                tc_fence_after();
                const bool ok = active && dk >= 0x1p-50f && dk < INFINITY && nqi >= 0x1p-60f;
                const u32 lim = min(w, ntiles - sp);   // positions in this batch
                auto valid = [&](int c) -> u32 {
                    return lim <= u32(32 * c) ? 0u : lim - u32(32 * c) >= 32 ? ~0u : (1u << (lim - u32(32 * c))) - 1u;
                };
#pragma unroll
                for (int c2 = 0; c2 < int(TC_TEST / 64); ++c2) {
                    if (u32(c2) * 64 >= w) break;   // block-uniform
                    u32 g0[32], g1[32];
                    tmem_ld32_start(acc + ((warp * 32u) << 16) + u32(c2 * 64), g0);
                    tmem_ld32_start(acc + ((warp * 32u) << 16) + u32(c2 * 64 + 32), g1);
                    tmem_wait2(g0, g1);
                    u32 sk0 = 0, sk1 = 0;   // positions this query can skip
#pragma unroll
                    for (int h = 0; h < 32; ++h) {
                        const float2 ra = S.trc[c2 * 64 + h], rb = S.trc[c2 * 64 + 32 + h];
                        const f32 la = __fmaf_rd(-2.0f, __uint_as_float(g0[h]), __fadd_rd(nql, ra.y));
                        const f32 lb = __fmaf_rd(-2.0f, __uint_as_float(g1[h]), __fadd_rd(nql, rb.y));
                        const f32 ta = __fadd_ru(sq, ra.x), tb = __fadd_ru(sq, rb.x);
                        sk0 |= u32(la > __fmul_ru(ta, ta) && la <= 3.4e38f) << h;
                        sk1 |= u32(lb > __fmul_ru(tb, tb) && lb <= 3.4e38f) << h;
                    }
                    const u32 mc0 = active ? valid(2 * c2) & (ok ? ~sk0 : ~0u) : 0u;
                    const u32 mc1 = active ? valid(2 * c2 + 1) & (ok ? ~sk1 : ~0u) : 0u;
                    if (c2 == 0) {
                        m0 = mc0;
                        m1 = mc1;
                    } else {
                        m2 = mc0;
                        m3 = mc1;
                    }
                }
                tc_fence_before();
            }
            {
                const u32 w0 = __reduce_or_sync(0xffffffffu, m0), w1 = __reduce_or_sync(0xffffffffu, m1);
                const u32 w2 = __reduce_or_sync(0xffffffffu, m2), w3 = __reduce_or_sync(0xffffffffu, m3);
                if (lane == 0) {
                    S.need[npar][warp][0] = w0;
                    S.need[npar][warp][1] = w1;
                    S.need[npar][warp][2] = w2;
                    S.need[npar][warp][3] = w3;
                }
            }
            __syncthreads();
            {
                const u32(&nd)[4][TC_TEST / 32] = S.need[npar];
                bm0 = nd[0][0] | nd[1][0] | nd[2][0] | nd[3][0];
                bm1 = nd[0][1] | nd[1][1] | nd[2][1] | nd[3][1];
                bm2 = nd[0][2] | nd[1][2] | nd[2][2] | nd[3][2];
                bm3 = nd[0][3] | nd[1][3] | nd[2][3] | nd[3][3];
                my0 = m0;
                my1 = m1;
                my2 = m2;
                my3 = m3;
            }
            npar ^= 1;
            bbase = sp;
            sp += w;
        };
        // next tile some query of the block needs (block-uniform); false when
        // the order is exhausted
        auto next_tile = [&](u32& T, bool& mine, u32 acc) -> bool {
            for (;;) {
                // lowest set position over the four words (no references to
                // the words: they stay in registers)
                if (bm0 | bm1 | bm2 | bm3) {
                    const u32 c = bm0 ? 0u : bm1 ? 1u : bm2 ? 2u : 3u;
                    const u32 bw = c == 0 ? bm0 : c == 1 ? bm1 : c == 2 ? bm2 : bm3;
                    const u32 myw = c == 0 ? my0 : c == 1 ? my1 : c == 2 ? my2 : my3;
                    const u32 b = u32(__ffs(bw) - 1);
                    const u32 rest = bw & (bw - 1);
                    if (c == 0) bm0 = rest;
                    else if (c == 1) bm1 = rest;
                    else if (c == 2) bm2 = rest;
                    else bm3 = rest;
                    T = spiral_tile(blk, bbase + c * 32 + b, ntiles);
                    mine = (myw >> b) & 1u;
                    return true;
                }
                if (sp >= ntiles) return false;
                refill(acc);
            }
        };

        u32 tl0 = 0, tl1 = 0, nbits = 0, nl = 0;   // stage tiles, this thread's need bits, tiles loaded
        for (int s = 0; s < NSTAGE; ++s) {
            u32 T;
            bool mine;
            if (!next_tile(T, mine, ~0u)) break;
            if (tid == 0) load_stage(s, T);
            if (s == 0) tl0 = T; else tl1 = T;
            nbits = (nbits & ~(1u << s)) | (u32(mine) << s);
            ++nl;
        }
        if (tid == 0) {
            mbar_wait(&S.bar_a, ph_a, err, &S.fail);
            mbar_wait(&S.bar_b[0], ub0 & 1, err, &S.fail);
            tc_fence_after();
            mma_tile(tmem, smem_addr(S.a), smem_addr(S.b[0]), smem_addr(S.aaug), smem_addr(S.pk[0] + PK_AUG),
                     smem_addr(S.zeros));
            mma_commit(&S.bar_mma[0]);
        }
        // every thread reads the query tile below: acquire its TMA phase
        mbar_wait(&S.bar_a, ph_a, err, &S.fail);
        ph_a ^= 1;
        u32 it = 0;
        for (; it < nl; ++it) {
            const int sb = int(it & 1);            // accumulator buffer
            const int st = int(it % NSTAGE);       // candidate stage
            mbar_wait(&S.bar_mma[sb], (sb ? um1 : um0) & 1, err, &S.fail);
            tc_fence_after();
            // every thread acquires the stage's (complete) TMA phase before
            // reading the candidate tile, its norm terms and ids
            mbar_wait(&S.bar_b[st], (st ? ub1 : ub0) & 1, err, &S.fail);
            const u32 T = st == 0 ? tl0 : tl1;
            const bool mine = (nbits >> st) & 1u;
            const u32 j0 = T * TC_N;
            if (__any_sync(0xffffffffu, mine)) {
                const unsigned char* bt = S.b[st];
                const u16* blo = reinterpret_cast<const u16*>(S.pk[st]);
                const u32* oid = reinterpret_cast<const u32*>(S.pk[st] + PK_ID);
                // Gram filter. D = G + w_hi + w_lo with G = q~ . c~ (TF32-exact
                // heads: exact products, FP32 accumulation, |G - q~.c~| <=
                // 2^-17 (|q~|^2 + |c~|^2)) and -w_hi - w_lo <= |c~|^2 (1 - 2^-16) / 2,
                // so L = nq (1 - 2^-16) - 2 D <= |q~ - c~|^2. A candidate that can
                // enter has |q - c| <= sqrt(T), and |q - c| >= |q~ - c~| - e_q - e_c
                // with e_c <= e_T (the tile's largest), so its L <= (sq + e_T)^2:
                // it passes iff D >= t = (nq (1 - 2^-16) - (sq + e_T)^2) / 2
                // (every step rounded toward passing).
                const float4 trec = *reinterpret_cast<const float4*>(S.pk[st] + PK_TAIL);
                const f32 eT = trec.z;
                const f32 sT = __fadd_ru(sq, eT);
                const f32 t = mine ? 0.5f * __fsub_rd(nql, __fmul_ru(sT, sT)) : INFINITY;
                // (A) filter the tile's 128 candidates, two 32-column TMEM loads
                // in flight at a time. Survivors are rare, so the common case is
                // a max-tree (three-input max, depth 3) per chunk; the bit mask
                // is built only by threads holding a survivor. Padding
                // candidates carry -3e38.
                auto filt = [&](const u32 (&v)[32], int chunk) -> u32 {
                    f32 h1[11];
#pragma unroll
                    for (int h = 0; h < 10; ++h)
                        h1[h] = fmax3(__uint_as_float(v[3 * h]), __uint_as_float(v[3 * h + 1]),
                                      __uint_as_float(v[3 * h + 2]));
                    h1[10] = fmaxf(__uint_as_float(v[30]), __uint_as_float(v[31]));
                    const f32 h2a = fmax3(h1[0], h1[1], h1[2]), h2b = fmax3(h1[3], h1[4], h1[5]);
                    const f32 h2c = fmax3(h1[6], h1[7], h1[8]), h2d = fmaxf(h1[9], h1[10]);
                    const f32 dmax = fmaxf(fmax3(h2a, h2b, h2c), h2d);
                    u32 m = 0;
                    if (active && dmax >= t) {
#pragma unroll
                        for (int h = 0; h < 32; ++h) m |= u32(__uint_as_float(v[h]) >= t) << h;
                        const u32 cbase = j0 + u32(chunk * 32);
                        // padding still passes while sq is +inf (list not yet full)
                        if (cbase + 32 > n) m &= cbase < n ? (1u << (n - cbase)) - 1u : 0u;
                        if (i >= cbase && i < cbase + 32) m &= ~(1u << (i - cbase));
                    }
                    return m;
                };
                u32 mk[TC_N / 32];
#pragma unroll
                for (int c2 = 0; c2 < TC_N / 64; ++c2) {
                    u32 v0[32], v1[32];
                    tmem_ld32_start(tmem + u32(sb) * TC_N + ((warp * 32u) << 16) + u32(c2 * 64), v0);
                    tmem_ld32_start(tmem + u32(sb) * TC_N + ((warp * 32u) << 16) + u32(c2 * 64 + 32), v1);
                    tmem_wait2(v0, v1);
                    mk[2 * c2] = filt(v0, 2 * c2);
                    mk[2 * c2 + 1] = filt(v1, 2 * c2 + 1);
                }
                // (B) survivors. Few per tile (after the first), spread over the
                // lanes: the warp queues its (query, candidate) pairs in shared
                // memory, every lane computes exact distances for its share of
                // the queue from the two resident tiles (query rows from the
                // swizzled query tile, candidates from the stage), and each
                // owner then inserts its own results. A queue longer than
                // TC_Q (the first tile of a block, while the lists fill) is
                // evaluated by the owners directly.
                const u32 tcnt = __popc(mk[0]) + __popc(mk[1]) + __popc(mk[2]) + __popc(mk[3]);
                const u32 total = __reduce_add_sync(0xffffffffu, tcnt);
                if (total > u32(TC_Q)) {
                    // Mostly the first tile of a block: the lists are empty and
                    // every candidate passed. The tile bounds its own k-th
                    // distance. For a candidate |q~ - c~|^2 <= (|q~|^2 + |c~|^2)
                    // (1 + 2^-16) - 2 (D - w_hi - w_lo) (the accumulation bound)
                    // and |c~|^2 + 2 (w_hi + w_lo) <= 2^-15.6 |c~|^2, so with N_T
                    // the tile's largest |c~|^2 (rounded down, as nq: within
                    // 2^-18), u = nq (1 + 2^-15) - 2 D + 2^-14 N_T >= |q~ - c~|^2
                    // (rounded up; a negative or NaN u, which only overflow can
                    // make, is no bound). The k-th smallest of 32 group minima of u (4
                    // candidates a group) is u of k distinct candidates, whose
                    // true distances are then <= sqrt(u_k) + e_q + e_T; with the
                    // lane-ordered sums' rounding, no candidate farther than
                    // s_B = (sqrt(u_k) + e_q + e_T) (1 + 2^-14) can enter, so one
                    // with L > (s_B + e_q + e_T)^2 is dropped.
                    {
                        f32 gm[32];
#pragma unroll
                        for (int chunk = 0; chunk < TC_N / 32; ++chunk) {
                            u32 v[32];
                            tmem_ld32(tmem + u32(sb) * TC_N + ((warp * 32u) << 16) + u32(chunk * 32), v);
#pragma unroll
                            for (int g = 0; g < 8; ++g) {
                                f32 d4[4];
#pragma unroll
                                for (int e = 0; e < 4; ++e)
                                    d4[e] = (mk[chunk] >> (4 * g + e)) & 1u ? __uint_as_float(v[4 * g + e]) : -INFINITY;
                                gm[chunk * 8 + g] = fmaxf(fmax3(d4[0], d4[1], d4[2]), d4[3]);
                            }
                        }
                        const f32 NT = trec.w;
                        const f32 au = __fmaf_ru(NT, 0x1p-14f, __fmul_ru(nqi, 1.0f + 0x1p-15f));
#pragma unroll
                        for (int g = 0; g < 32; ++g) {
                            const f32 u = __fmaf_ru(-2.0f, gm[g], au);
                            gm[g] = u >= 0.0f ? u : INFINITY;   // no candidate in the group: +inf
                        }
                        bitonic_sort<32>(gm);
                        // B = gm[k - 1] by a bit-mask select (an opaque mask, so the
                        // compiler keeps gm in registers instead of indexing it)
                        u32 ksel = 1u << (k - 1);
                        asm volatile("" : "+r"(ksel));
                        f32 B = INFINITY;
#pragma unroll
                        for (int g = 0; g < TC_K; ++g) B = (ksel >> g) & 1u ? gm[g] : B;
                        const f32 sB = __fmul_ru(__fadd_ru(__fadd_ru(__fsqrt_ru(B), eqi), eT), 1.0f + 0x1p-14f);
                        const f32 sB2 = __fadd_ru(__fadd_ru(sB, eqi), eT);
                        // (relative bounds: |q|^2 far above the subnormal range)
                        const f32 t2 = B < INFINITY && nqi >= 0x1p-60f ? 0.5f * __fsub_rd(nql, __fmul_ru(sB2, sB2))
                                                                      : -INFINITY;
                        if (__any_sync(0xffffffffu, t2 > t)) {
                            const f32 tt = fmaxf(t, t2);
#pragma unroll 1
                            for (int chunk = 0; chunk < TC_N / 32; ++chunk) {
                                u32 v[32];
                                tmem_ld32(tmem + u32(sb) * TC_N + ((warp * 32u) << 16) + u32(chunk * 32), v);
                                u32 m = 0;
#pragma unroll
                                for (int h = 0; h < 32; ++h) m |= u32(__uint_as_float(v[h]) >= tt) << h;
                                mk[0] &= chunk == 0 ? m : ~0u;   // constant indices keep mk in registers
                                mk[1] &= chunk == 1 ? m : ~0u;
                                mk[2] &= chunk == 2 ? m : ~0u;
                                mk[3] &= chunk == 3 ? m : ~0u;
                            }
                        }
                    }
                    bool changed = false;
                    f32 qa[TC_DIM];   // this thread's query, from the query tile
                    raw_row(S.a, S.alo, row, qa);
                    u32 m0 = mk[0], m1 = mk[1], m2 = mk[2], m3 = mk[3];
#pragma unroll 1
                    while (m0 | m1 | m2 | m3) {   // one pass over the set bits
                        const u32 c = m0 ? 0u : m1 ? 32u : m2 ? 64u : 96u;
                        const u32 wd = m0 ? m0 : m1 ? m1 : m2 ? m2 : m3;
                        const u32 rr = c + u32(__ffs(wd) - 1);
                        const u32 rest = wd & (wd - 1);
                        if (m0) m0 = rest;
                        else if (m1) m1 = rest;
                        else if (m2) m2 = rest;
                        else m3 = rest;
                        f32 cb[TC_DIM];
                        raw_row(bt, blo, rr, cb);
                        changed |= consider(oid[rr], __fsqrt_rn(l2_sq_acc(RegVec<TC_DIM>{qa}, RegVec<TC_DIM>{cb}, TC_DIM)));
                    }
                    if (changed) update_bound();
                } else if (total) {
                    u32 incl = tcnt;   // queue positions: an inclusive scan of the counts
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const u32 y = __shfl_up_sync(0xffffffffu, incl, o);
                        if (lane >= u32(o)) incl += y;
                    }
                    const u32 base = incl - tcnt;
                    u32* wq = S.q[warp];
                    f32* wr = S.r[warp];
                    {   // this lane's survivors into the queue: one pass over the set bits
                        u32 m0 = mk[0], m1 = mk[1], m2 = mk[2], m3 = mk[3];
                        u32 pos = base;
#pragma unroll 1
                        while (m0 | m1 | m2 | m3) {
                            const u32 c = m0 ? 0u : m1 ? 32u : m2 ? 64u : 96u;
                            const u32 wd = m0 ? m0 : m1 ? m1 : m2 ? m2 : m3;
                            wq[pos++] = (lane << 7) | (c + u32(__ffs(wd) - 1));
                            const u32 rest = wd & (wd - 1);
                            if (m0) m0 = rest;
                            else if (m1) m1 = rest;
                            else if (m2) m2 = rest;
                            else m3 = rest;
                        }
                    }
                    __syncwarp();
#pragma unroll 1
                    for (u32 p = lane; p < total; p += 32) {
                        const u32 e = wq[p];
                        f32 qa[TC_DIM], cb[TC_DIM];
                        raw_row(S.a, S.alo, warp * 32 + (e >> 7), qa);
                        raw_row(bt, blo, e & 127u, cb);
                        wr[p] = __fsqrt_rn(l2_sq_acc(RegVec<TC_DIM>{qa}, RegVec<TC_DIM>{cb}, TC_DIM));
                    }
                    __syncwarp();
                    bool changed = false;
#pragma unroll 1
                    for (u32 kk = 0; kk < tcnt; ++kk)
                        changed |= consider(oid[wq[base + kk] & 127u], wr[base + kk]);
                    if (changed) update_bound();
                    __syncwarp();   // the queue is reused by the next tile
                }
            }
            // the next tile's product, issued by the first warp whose epilogue
            // is done (its copy has had that epilogue to land; accumulator nb
            // and stage ns were released at the last barrier); the tensor
            // core runs it while the other warps finish this tile. The last
            // warp to arrive resets the parity's ticket, which is next used
            // two tiles on, after a barrier.
            if (it + 1 < nl) {
                u32 order = 0;
                if (lane == 0) order = atomicAdd(&S.ticket[it & 1], 1u);
                order = __shfl_sync(0xffffffffu, order, 0);
                if (order == 3 && lane == 0) S.ticket[it & 1] = 0;
                if (order == 0 && lane == 0) {
                    const int nb = sb ^ 1, ns = int((it + 1) % NSTAGE);
                    mbar_wait(&S.bar_b[ns], (ns ? ub1 : ub0) & 1, err, &S.fail);
                    tc_fence_after();
                    mma_tile(tmem + u32(nb) * TC_N, smem_addr(S.a), smem_addr(S.b[ns]), smem_addr(S.aaug),
                             smem_addr(S.pk[ns] + PK_AUG), smem_addr(S.zeros));
                    mma_commit(&S.bar_mma[nb]);
                }
            }
            if (sb) ++um1; else ++um0;
            // one reader of this CTA's timeout flag (shared memory: a global
            // poll here would put an L2 round trip on every tile); the
            // decision is double-buffered by tile parity, so the write for
            // tile it + 2 cannot overtake a read of this one
            if (tid == 0) S.stop[it & 1] = S.fail;
            tc_fence_before();
            __syncthreads();   // TMEM buffer sb and shared stage st are free again
            if (st) ++ub1; else ++ub0;
            if (S.stop[it & 1]) {   // block-uniform
                failed = true;
                break;
            }
            u32 Tn;
            bool mn;
            if (next_tile(Tn, mn, tmem + u32(sb) * TC_N)) {   // block-uniform (may test a batch)
                if (tid == 32) {   // warp 1 issues the copies, warp 0 the products
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    load_stage(st, Tn);
                }
                if (st == 0) tl0 = Tn; else tl1 = Tn;
                nbits = (nbits & ~(1u << st)) | (u32(mn) << st);
                ++nl;
            }
        }
        if (failed) {
            // bounded drain of what is still in flight: the product and the
            // copy of tile it + 1 (no copy was issued after the failure showed)
            if (tid == 0) {
                const u32 u1 = (it + 1) & 1;
                if (it + 1 < nl) mbar_wait(&S.bar_mma[u1], (u1 ? um1 : um0) & 1, nullptr);
                for (u32 u = it + 1; u < nl; ++u) mbar_wait(&S.bar_b[u & 1], ((u & 1) ? ub1 : ub0) & 1, nullptr);
                // the last lookahead product (returns at once if it completed)
                if (ut) mbar_wait(&S.bar_t, (ut - 1) & 1, nullptr);
            }
            __syncthreads();
            break;
        }
        tiles_done += nl;
        if (active) {
            const u32 oi = reinterpret_cast<const u32*>(pack + u64(blk) * PACK_BYTES + PK_ID)[row];
            const u32 first = TC_K - k;   // entries [first, TC_K) are the k results
#pragma unroll
            for (int s = 0; s < TC_K; ++s)
                if (u32(s) >= first) {
                    ids[u64(oi) * k + (s - first)] = u32(lk[s]);
                    if (dists) dists[u64(oi) * k + (s - first)] = __uint_as_float(u32(lk[s] >> 32));
                }
        }
        __syncthreads();
    }
    if (counters) {   // one atomic a warp
        unsigned long long ev = exact_evals;
#pragma unroll
        for (int o = 16; o; o >>= 1) ev += __shfl_xor_sync(0xffffffffu, ev, o);
        if (lane == 0 && ev) atomicAdd(&counters[0], ev);
        if (tid == 0 && tiles_done) atomicAdd(&counters[1], tiles_done);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TC_N) : "memory");
}

// ---- a check of the tensor core's accumulation bound ------------------------
//
// The Gram filter's margins are derived for an accumulation error of at
// most 2^-17 (|a|^2 + |b|^2) over the five K-steps (32 coordinates and the
// augmentation) of kind::tf32 with FP32 accumulation on TF32-exact operands
// (the accumulation bound at the top of this file). This kernel measures
// that error on the device: one 128 x 128 product per CTA of seeded
// TF32-exact rows (mixed exponents 2^-8 .. 2^8 and signs, and rows near a
// common offset, where the sum cancels), issued exactly as the kNN kernel
// issues it, against an FP64 sum of the same products. out: the largest
// |D - exact| / (|a|^2 + |b|^2), as the bits of a non-negative double.
struct GramCheckSmem {
    alignas(1024) float4 aaug[TC_M];
    float4 baug[TC_N];
    float4 zeros[TC_N];
    alignas(1024) unsigned char a[TILE_BYTES];
    alignas(1024) unsigned char b[TILE_BYTES];
    alignas(8) u64 bar;
    u32 tmem_base;
};
constexpr size_t GC_SMEM = 72 * 1024;   // at most three CTAs an SM: 3 x 128 TMEM columns
static_assert(sizeof(GramCheckSmem) + 1024 <= GC_SMEM, "check layout exceeds its reservation");

__device__ __forceinline__ u32 gc_hash(u64 x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return u32(x);
}

// coordinate k of row r of operand side (0 = queries, 1 = candidates) in product t
__device__ __forceinline__ f32 gc_value(u64 seed, u32 t, u32 side, u32 r, u32 k) {
    const u32 h = gc_hash(seed ^ (u64(t) << 40) ^ (u64(side) << 39) ^ (u64(r) << 8) ^ k);
    const u32 rowkind = gc_hash(seed ^ (u64(t) << 40) ^ (u64(side) << 39) ^ (u64(r) << 8) ^ 0xffu) & 3u;
    if (rowkind == 0) {   // near a common offset of 100: the Gram sum cancels against the norms
        const f32 off = 100.0f + f32(int(h & 1023u) - 512) * 0x1p-10f;
        return __uint_as_float(__float_as_uint(off) & 0xffffe000u);
    }
    const int e = int((h >> 10) % 17u) - 8;               // 2^-8 .. 2^8
    const f32 mant = 1.0f + f32(h & 1023u) * 0x1p-10f;    // 11 significant bits: TF32-exact
    const f32 v = ldexpf(mant, e);
    return (h >> 31) ? -v : v;
}

__global__ void __launch_bounds__(128) k_tc_gram_check(u64 seed, unsigned long long* __restrict__ out,
                                                      u32* __restrict__ err) {
    extern __shared__ unsigned char gc_raw[];
    GramCheckSmem& S = *reinterpret_cast<GramCheckSmem*>((reinterpret_cast<uintptr_t>(gc_raw) + 1023) & ~uintptr_t(1023));
    const u32 tid = threadIdx.x, warp = tid >> 5, t = blockIdx.x;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&S.tmem_base)),
                     "r"(TC_N)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    // this thread's query row and candidate row, swizzled as the TMA writes them
    f32 qa[TC_DIM], cb[TC_DIM];
    f32 nb = 0.0f;
#pragma unroll
    for (int k = 0; k < TC_DIM; ++k) {
        qa[k] = gc_value(seed, t, 0, tid, u32(k));
        cb[k] = gc_value(seed, t, 1, tid, u32(k));
        nb = __fmaf_rd(cb[k], cb[k], nb);
    }
#pragma unroll
    for (int ch = 0; ch < 8; ++ch) {
        *reinterpret_cast<float4*>(S.a + tid * 128 + ((ch ^ (tid & 7)) << 4)) =
            make_float4(qa[4 * ch], qa[4 * ch + 1], qa[4 * ch + 2], qa[4 * ch + 3]);
        *reinterpret_cast<float4*>(S.b + tid * 128 + ((ch ^ (tid & 7)) << 4)) =
            make_float4(cb[4 * ch], cb[4 * ch + 1], cb[4 * ch + 2], cb[4 * ch + 3]);
    }
    {   // the augmentation rows, made as the regrouping makes them
        const f32 w = -__fmul_rd(nb, 0.5f * (1.0f - 0x1p-16f));
        const f32 hi = __uint_as_float(__float_as_uint(w) & 0xffffe000u);
        const f32 lo = __uint_as_float(__float_as_uint(w - hi) & 0xffffe000u);
        S.aaug[tid] = make_float4(1.0f, 1.0f, 0.0f, 0.0f);
        S.baug[tid] = make_float4(hi, lo, 0.0f, 0.0f);
        S.zeros[tid] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    if (tid == 0) {
        mbar_init(&S.bar, 1);
        fence_mbar_init();
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const u32 tmem = S.tmem_base;
    if (tid == 0) {
        mma_tile(tmem, smem_addr(S.a), smem_addr(S.b), smem_addr(S.aaug), smem_addr(S.baug), smem_addr(S.zeros));
        mma_commit(&S.bar);
    }
    mbar_wait(&S.bar, 0, err);
    tc_fence_after();
    double na = 0.0;
#pragma unroll
    for (int k = 0; k < TC_DIM; ++k) na += double(qa[k]) * double(qa[k]);
    double worst = 0.0;
#pragma unroll 1
    for (int chunk = 0; chunk < TC_N / 32; ++chunk) {
        u32 v[32];
        tmem_ld32(tmem + ((warp * 32u) << 16) + u32(chunk * 32), v);
#pragma unroll 1
        for (int h = 0; h < 32; ++h) {
            const u32 c = u32(chunk * 32 + h);
            f32 cr[TC_DIM];
            swz_row(S.b, c, cr);
            double dot = 0.0, ncr = 0.0;
#pragma unroll
            for (int k = 0; k < TC_DIM; ++k) {
                dot += double(qa[k]) * double(cr[k]);
                ncr += double(cr[k]) * double(cr[k]);
            }
            const float4 au = S.baug[c];
            const double exact = dot + double(au.x) + double(au.y);
            const double r = fabs(double(__uint_as_float(v[h])) - exact) / (na + ncr);
            worst = r > worst ? r : worst;
        }
    }
    atomicMax(out, (unsigned long long)__double_as_longlong(worst));
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_N) : "memory");
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        TT_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
        if (!p || q != cudaDriverEntryPointSuccess) throw Error(TT_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
        fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

}  // namespace

// The largest measured |D - exact| / (|a|^2 + |b|^2) over `products` seeded
// 128 x 128 tensor-core products (see k_tc_gram_check).
double tc_gram_check(tt_ctx* c, u32 products, u64 seed) {
    unsigned long long* out = c->arena.get<unsigned long long>(S_MISC1, 2);
    u32* err = reinterpret_cast<u32*>(out + 1);
    TT_CUDA(cudaMemsetAsync(out, 0, 2 * sizeof(unsigned long long), c->stream));
    TT_CUDA(cudaFuncSetAttribute(k_tc_gram_check, cudaFuncAttributeMaxDynamicSharedMemorySize, int(GC_SMEM)));
    if (products) {
        k_tc_gram_check<<<products, 128, GC_SMEM, c->stream>>>(seed, out, err);
        TT_LAUNCH("k_tc_gram_check");
        ++c->launches;
    }
    unsigned long long h[2] = {0, 0};
    TT_CUDA(cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    TT_CUDA(cudaStreamSynchronize(c->stream));
    if (u32(h[1])) throw Error(TT_ERR_TIMEOUT, "gb300: a bounded device wait timed out in the Gram check");
    double r;
    __builtin_memcpy(&r, &h[0], sizeof(r));
    return r;
}

bool knn_tc_applicable(u32 n, u32 dim, int kind, u32 k, const f32* x) {
    return kind == M_L2 && dim == u32(TC_DIM) && k >= 1 && k <= u32(TC_K) && n >= 2 &&
           (reinterpret_cast<uintptr_t>(x) & 15) == 0;
}

// The deferred status of the last knn_tc (error word, counters), once the
// stream has been synchronised: throws on a device timeout.
void knn_tc_settle(tt_ctx* c) {
    if (!c->tc_pending) return;
    c->tc_pending = false;
    if (c->tc_host[0]) throw Error(TT_ERR_TIMEOUT, "gb300: a bounded device wait timed out in the tensor-core kNN");
    c->filter_evals = c->tc_host[1];
    c->filter_tiles = c->tc_host[2];
}

// Exact kNN lists through the tile order and the tensor-core filter; sets
// the context's counts of exact evaluations and computed Gram tiles. With
// defer, the status is only copied back: the caller synchronises later and
// then calls knn_tc_settle before it relies on the lists.
// Slots: S_TC_* (regrouped heads, tile packs, error terms, tile records), S_MISC0/1, S_COUNT, and
// the radix sort's own (S_SORT_*, S_SCAN*).
void knn_tc(tt_ctx* c, const f32* x, u32 n, u32 k, u32* ids, f32* dists, bool defer) {
    const u32 ntiles = div_up(n, TC_N);
    const u64 wpad = u64(ntiles) * TC_N;
    // about 12 tiles per pivot region
    const u32 P = std::max<u32>(1, std::min<u32>(MAX_PIV, n / (12 * TC_N)));
    u32* perm = nullptr;
    {
        f32* piv = c->arena.get<f32>(S_TC_PIV, u64(P) * TC_DIM + MAX_PIV);
        u32* rank = reinterpret_cast<u32*>(piv + u64(P) * TC_DIM);
        u64* key = c->arena.get<u64>(S_TC_KEYS, n);
        u32* val = c->arena.get<u32>(S_TC_VALS, n);
        const size_t psmem = (size_t(P) * (TC_DIM + 1) + size_t(P) * P) * sizeof(f32);
        TT_CUDA(cudaFuncSetAttribute(k_tc_pivots, cudaFuncAttributeMaxDynamicSharedMemorySize, int(psmem)));
        {   // the pivot chain (one CTA) on the side stream, beside the assignment
            SideScope side(c);
            const cudaStream_t ps = side.fork();
            k_tc_pivots<<<1, PIV_THREADS, psmem, ps>>>(x, n, P, piv, rank);
            TT_LAUNCH("k_tc_pivots");
            launch_pdl(k_tc_assign, div_up(div_up(n, 2), 256), 256, P * (TC_DIM + 1) * sizeof(f32), c->stream, x, n, P,
                       key, val);
            TT_LAUNCH("k_tc_assign");
            side.join();
        }
        k_tc_rank<<<std::min<u32>(div_up(n, 256), 4 * u32(c->sms)), 256, 0, c->stream>>>(rank, n, key);
        TT_LAUNCH("k_tc_rank");
        c->launches += 1;
        c->launches += 2;
        perm = val;
        u64* skey = key;
        u64* kb = c->arena.get<u64>(S_SORT_A, n);
        u32* vb = c->arena.get<u32>(S_SORT_VA, n);
        const int bits = P > 1 ? 32 - __builtin_clz(P - 1) : 0;
        if (P > 1 && radix_sort<u32>(c, key, val, n, kb, vb, bits)) {
            perm = vb;
            skey = kb;
        }
        // second level: sub-cells within every cell (tiles then follow them)
        if (n >= 2 * TC_N) {
            u32* cell_off = c->arena.get<u32>(S_TC_CELL, u64(P) + 2);
            u64* key2 = c->arena.get<u64>(S_TC_KEY2, n);
            u32* val2 = c->arena.get<u32>(S_TC_VAL2, n);
            launch_pdl(k_tc_cells, 1, 256, 0, c->stream, skey, n, P, cell_off);
            TT_LAUNCH("k_tc_cells");
            f32* spv = c->arena.get<f32>(S_TC_SPV, u64(P) * 16 * (TC_DIM + 1));
            f32* spn = spv + u64(P) * 16 * TC_DIM;
            launch_pdl(k_tc_subpiv, div_up(u64(P) * 16 * 32, 256), 256, 0, c->stream, x, perm, cell_off, P, spv, spn);
            TT_LAUNCH("k_tc_subpiv");
            launch_pdl(k_tc_assign2, div_up(n, 256), 256, 0, c->stream, x, n, skey, perm, cell_off, spv, spn, key2, val2);
            TT_LAUNCH("k_tc_assign2");
            c->launches += 3;
            perm = radix_sort<u32>(c, key2, val2, n, kb, vb, bits + 4) ? vb : val2;
        }
    }
    f32* xh = c->arena.get<f32>(S_TC_X, u64(n) * TC_DIM);
    unsigned char* pack = c->arena.get<unsigned char>(S_TC_LO, u64(ntiles) * PACK_BYTES);
    f32* eq = c->arena.get<f32>(S_TC_ERR, wpad);
    f32* nq = c->arena.get<f32>(S_MISC0, wpad);
    f32* stats = c->arena.get<f32>(S_TC_STATS, u64(ntiles) * ST_STRIDE);
    u32* ctl = c->arena.get<u32>(S_MISC1, 4);   // [0] next block, [1] error word
    unsigned long long* cnt = c->arena.get<unsigned long long>(S_COUNT, 2);
    TT_CUDA(cudaMemsetAsync(ctl, 0, 4 * sizeof(u32), c->stream));
    TT_CUDA(cudaMemsetAsync(cnt, 0, 2 * sizeof(unsigned long long), c->stream));
    launch_pdl(k_tc_tiles, ntiles, TC_N, 0, c->stream, x, n, perm, xh, pack, nq, eq, stats);
    TT_LAUNCH("k_tc_tiles");
    CUtensorMap map;
    const cuuint64_t gdim[2] = {cuuint64_t(TC_DIM), cuuint64_t(n)};
    const cuuint64_t gstride[1] = {cuuint64_t(TC_DIM) * 4};
    const cuuint32_t box[2] = {cuuint32_t(TC_DIM), cuuint32_t(TC_M)};
    const cuuint32_t estride[2] = {1, 1};
    const CUresult r = encode_fn()(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, xh, gdim, gstride, box, estride,
                                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw Error(TT_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string(int(r)) + ")");
    TT_CUDA(cudaFuncSetAttribute(k_knn_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, int(TC_SMEM)));
    const u32 grid = std::min<u32>(ntiles, 2 * u32(c->sms));
    launch_pdl(k_knn_tc, grid, 128, TC_SMEM, c->stream, map, pack, eq, n, k, nq, stats, ids, dists, ctl, ctl + 1, cnt);
    TT_LAUNCH("k_knn_tc");
    c->launches += 2;
    if (!c->tc_host) TT_CUDA(cudaMallocHost(&c->tc_host, 4 * sizeof(unsigned long long)));
    c->tc_host[0] = 0;
    TT_CUDA(cudaMemcpyAsync(c->tc_host, ctl + 1, 4, cudaMemcpyDeviceToHost, c->stream));
    TT_CUDA(cudaMemcpyAsync(c->tc_host + 1, cnt, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream));
    c->tc_pending = true;
    if (!defer) {
        TT_CUDA(cudaStreamSynchronize(c->stream));
        knn_tc_settle(c);
    }
}

}  // namespace tt
