// tt_knn_tc.cu — exact L2 k nearest neighbours in R^32 with a tensor-core
// (tcgen05) Gram filter.
//
// Same result as the exhaustive scan (tt_scan.cuh KnnOp, which replaces
// graph.hpp knn_lists_exact :211-225): the k smallest (distance, id) pairs
// per query, every distance the reference's lane-ordered float32 l2
// (metric.hpp:92-112). The Gram product only decides which candidates are
// worth that exact evaluation:
//
//   s~(q, c) = |q|^2 + |c|^2 - 2 G~(q, c),   G~ = TF32 tensor-core Gram, FP32 sum
//
// TF32 keeps 10 mantissa bits of each operand, so |G~ - q.c| <= 2^-9 |q||c|
// <= 2^-10 (|q|^2 + |c|^2); with the FP32 norms and the final fma the error of
// s~ stays below 2^-8 (|q|^2 + |c|^2). A candidate is evaluated exactly when
//
//   s~ - 2^-7 (|q|^2 + |c|^2) <= T_q,   T_q = sq_bound(d_k) (1 + 2^-16)
//
// where d_k is the query's current k-th exact distance: every candidate
// whose exact distance could enter the list passes (the 2^-16 covers the
// lane-ordered sum's own rounding), so the filter never changes a result.
//
// Pipeline per CTA (128 threads = 4 warps, one query row per thread, 128
// queries per block, persistent over query blocks):
//   TMA (cp.async.bulk.tensor, 128-byte swizzle) loads the query tile once
//   and candidate tiles of 128 points into two shared-memory stages;
//   thread 0 issues tcgen05.mma.kind::tf32 (M = 128, N = 128, 4 x K = 8)
//   into one of two TMEM accumulators and commits to an mbarrier; while
//   the tensor core works on tile t + 1 the four warps read tile t's Gram
//   rows (tcgen05.ld 32x32b.x32), run the filter and the exact path.
// TMEM: 2 x 128 columns per CTA; shared memory is padded so that at most two
// CTAs share an SM, so tcgen05.alloc never waits. Every mbarrier wait is
// bounded (tt_tma.cuh); on a timeout the kernel records the error, stops,
// and still frees its TMEM.
#include <cuda.h>

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
constexpr int TC_BUF = 16;                      // deferred survivors per thread
constexpr int NSTAGE = 2;                       // candidate tiles in flight (TMA ring)
constexpr size_t TC_SMEM = 100 * 1024;          // caps residency at two CTAs per SM

constexpr u32 WC_BYTES = TC_N * 4;               // candidate norm terms per tile

struct Shared {
    alignas(1024) unsigned char a[TILE_BYTES];
    alignas(1024) unsigned char b[NSTAGE][TILE_BYTES];
    alignas(16) f32 wcs[NSTAGE][TC_N];                // |c|^2 (1 - 2^-7) of the tile's candidates
    u32 buf[16][128];                            // deferred survivors, entry-major (conflict-free)
    alignas(8) u64 bar_a;
    alignas(8) u64 bar_b[NSTAGE];
    alignas(8) u64 bar_mma[2];
    u32 tmem_base;
    u32 block;
    u32 stop;
};

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

// UMMA shared-memory descriptor: K-major operand, 128-byte swizzle, rows of
// 128 bytes in 1024-byte groups of 8 (stride byte offset 1024), version 1.
__device__ __forceinline__ u64 sw128_desc(u32 saddr) {
    return u64((saddr >> 4) & 0x3fff) | (u64(1) << 16) | (u64(1024 >> 4) << 32) | (u64(1) << 46) |
           (u64(2) << 61);
}

// Instruction descriptor, kind::tf32: D f32, A/B tf32, both K-major, N, M.
constexpr u32 kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | (u32(TC_N >> 3) << 17) | (u32(TC_M >> 4) << 24);

__device__ __forceinline__ void tma_tile(void* dst, const CUtensorMap* map, int row, u64* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(smem_addr(dst)),
        "l"(map), "r"(0), "r"(row), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void mma_tile(u32 d_tmem, u32 a_saddr, u32 b_saddr) {
#pragma unroll
    for (int ks = 0; ks < TC_DIM / 8; ++ks) {   // K = 8 tf32 = 32 bytes per step
        const u64 da = sw128_desc(a_saddr + 32 * ks);
        const u64 db = sw128_desc(b_saddr + 32 * ks);
        const u32 acc = ks > 0;
        asm volatile(
            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
            "l"(da), "l"(db), "r"(kIdesc), "r"(acc)
            : "memory");
    }
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

__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

template <int DIM>
struct RegVec {
    const f32 (&q)[DIM];
    __device__ __forceinline__ f32 operator()(u32 k) const { return q[k]; }
};

// |x_i|^2 and the filter's candidate term |x_i|^2 (1 - 2^-7); padding
// candidates (i in [n, wpad)) get +inf so that they never pass the filter.
__global__ void k_norms(const f32* __restrict__ x, u32 n, u32 wpad, f32* __restrict__ nq, f32* __restrict__ wc) {
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < wpad; i += gridDim.x * blockDim.x) {
        if (i >= n) {
            wc[i] = INFINITY;
            continue;
        }
        f32 s = 0.0f;
#pragma unroll
        for (int k = 0; k < TC_DIM; ++k) s = fmaf(x[u64(i) * TC_DIM + k], x[u64(i) * TC_DIM + k], s);
        nq[i] = s;
        wc[i] = s * (1.0f - 1.0f / 128.0f);
    }
}

__global__ void __launch_bounds__(128, 2)
k_knn_tc(const __grid_constant__ CUtensorMap map, const f32* __restrict__ x, u32 n, u32 k,
         const f32* __restrict__ nq, const f32* __restrict__ wc, u32* __restrict__ ids, f32* __restrict__ dists,
         u32* __restrict__ next_block, u32* __restrict__ err, unsigned long long* __restrict__ exact_count) {
    extern __shared__ unsigned char smem_raw[];
    Shared& S = *reinterpret_cast<Shared*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const u32 tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const u32 nblocks = (n + TC_M - 1) / TC_M;
    const u32 ntiles = (n + TC_N - 1) / TC_N;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&S.tmem_base)),
                     "r"(2 * TC_N)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        mbar_init(&S.bar_a, 1);
        for (int q = 0; q < NSTAGE; ++q) mbar_init(&S.bar_b[q], 1);
        mbar_init(&S.bar_mma[0], 1);
        mbar_init(&S.bar_mma[1], 1);
        fence_mbar_init();
        S.stop = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const u32 tmem = S.tmem_base;
    u32 ph_a = 0, uses_b[NSTAGE] = {}, uses_mma[2] = {0, 0};
    unsigned long long exact_evals = 0;
    bool failed = false;

    // stage s <- candidate tile t: the points (TMA, swizzled) and their norm terms
    auto load_stage = [&](int s, u32 t) {
        mbar_expect_tx(&S.bar_b[s], TILE_BYTES + WC_BYTES);
        tma_tile(S.b[s], &map, int(t * TC_N), &S.bar_b[s]);
        bulk_g2s(S.wcs[s], wc + u64(t) * TC_N, WC_BYTES, &S.bar_b[s]);
    };

    for (;;) {
        if (tid == 0) S.block = atomicAdd(next_block, 1u);
        __syncthreads();
        const u32 blk = S.block;
        if (blk >= nblocks || failed) break;
        const u32 q0 = blk * TC_M;
        if (tid == 0) {
            mbar_expect_tx(&S.bar_a, TILE_BYTES);
            tma_tile(S.a, &map, int(q0), &S.bar_a);
            for (u32 t = 0; t < u32(NSTAGE) && t < ntiles; ++t) load_stage(int(t), t);
        }
        const u32 row = warp * 32 + lane;
        const u32 i = q0 + row;
        const bool active = i < n;
        const f32 nqi = active ? nq[i] : 0.0f;
        f32 q[TC_DIM];
#pragma unroll
        for (int c = 0; c < TC_DIM; ++c) q[c] = active ? x[u64(i) * TC_DIM + c] : 0.0f;
        f32 ld[TC_K];
        u32 lj[TC_K];
#pragma unroll
        for (int t = 0; t < TC_K; ++t) {
            ld[t] = INFINITY;
            lj[t] = 0xffffffffu;
        }
        f32 rq = INFINITY;   // candidate passes iff fma(-2, G, wc) <= rq
        u32 nbuf = 0;        // deferred survivors of this thread (S.buf[.][tid])
        // insert (d, j) into the sorted top-TC_K list; true if it entered
        auto consider = [&](u32 j, f32 d) -> bool {
            ++exact_evals;
            if (!(d < ld[TC_K - 1] || (d == ld[TC_K - 1] && j < lj[TC_K - 1]))) return false;
            bool placed = false;
#pragma unroll
            for (int s = TC_K - 1; s >= 1; --s) {
                if (!placed) {
                    if (d < ld[s - 1] || (d == ld[s - 1] && j < lj[s - 1])) {
                        ld[s] = ld[s - 1];
                        lj[s] = lj[s - 1];
                    } else {
                        ld[s] = d;
                        lj[s] = j;
                        placed = true;
                    }
                }
            }
            if (!placed) {
                ld[0] = d;
                lj[0] = j;
            }
            return true;
        };
        // filter bound from the k-th entry; +inf until the list holds k
        auto update_rq = [&]() {
            f32 dk = INFINITY;
#pragma unroll
            for (int s = 0; s < TC_K; ++s)
                if (s == int(k) - 1) dk = ld[s];
            const f32 tq = dk < INFINITY ? sq_bound(dk) * (1.0f + 1.0f / 65536.0f) : INFINITY;
            rq = tq - nqi * (1.0f - 1.0f / 128.0f);
        };
        // evaluate the deferred survivors (coordinates from global memory / L2)
        auto flush = [&]() {
            bool changed = false;
#pragma unroll 1
            for (u32 e = 0; e < nbuf; ++e) {
                const u32 j = S.buf[e][tid];
                const float4* xr = reinterpret_cast<const float4*>(x + u64(j) * TC_DIM);
                f32 cb[TC_DIM];
#pragma unroll
                for (int ch = 0; ch < 8; ++ch) {
                    const float4 t4 = __ldg(xr + ch);
                    cb[4 * ch] = t4.x;
                    cb[4 * ch + 1] = t4.y;
                    cb[4 * ch + 2] = t4.z;
                    cb[4 * ch + 3] = t4.w;
                }
                changed |= consider(j, __fsqrt_rn(l2_sq_acc(RegVec<TC_DIM>{q}, RegVec<TC_DIM>{cb}, TC_DIM)));
            }
            nbuf = 0;
            if (changed) update_rq();
        };
        if (tid == 0) {
            mbar_wait(&S.bar_a, ph_a, err);
            mbar_wait(&S.bar_b[0], uses_b[0] & 1, err);
            tc_fence_after();
            mma_tile(tmem, smem_addr(S.a), smem_addr(S.b[0]));
            mma_commit(&S.bar_mma[0]);
        }
        // every thread reads the query tile below: acquire its TMA phase
        mbar_wait(&S.bar_a, ph_a, err);
        ph_a ^= 1;
        for (u32 t = 0; t < ntiles; ++t) {
            const int sb = int(t & 1);            // accumulator buffer
            const int st = int(t % NSTAGE);       // candidate stage
            mbar_wait(&S.bar_mma[sb], uses_mma[sb] & 1, err);
            tc_fence_after();
            if (tid == 0 && t + 1 < ntiles) {   // the tensor core works on t + 1 during this epilogue
                const int nb = sb ^ 1, ns = int((t + 1) % NSTAGE);
                mbar_wait(&S.bar_b[ns], uses_b[ns] & 1, err);   // tile t+1's phase (issued NSTAGE-1 tiles ago)
                tc_fence_after();
                mma_tile(tmem + u32(nb) * TC_N, smem_addr(S.a), smem_addr(S.b[ns]));
                mma_commit(&S.bar_mma[nb]);
            }
            // every thread acquires the stage's (complete) TMA phase before
            // reading the candidate tile and its norm terms
            mbar_wait(&S.bar_b[st], uses_b[st] & 1, err);
            const u32 j0 = t * TC_N;
            const unsigned char* bt = S.b[st];
            const f32* wcs = S.wcs[st];
            // (A) filter the tile's 128 candidates, 32 per TMEM load. Survivors
            // are rare, so the common case is a min-tree (32 independent fmas,
            // depth-5 fminf) per chunk; the bit mask is built only by threads
            // holding a survivor. Padding candidates carry +inf terms.
            u32 mk[TC_N / 32];
#pragma unroll
            for (int chunk = 0; chunk < TC_N / 32; ++chunk) {
                u32 v[32];
                tmem_ld32(tmem + u32(sb) * TC_N + ((warp * 32u) << 16) + u32(chunk * 32), v);
                f32 e[32];
#pragma unroll
                for (int g = 0; g < 8; ++g) {
                    const float4 w4 = *reinterpret_cast<const float4*>(wcs + chunk * 32 + 4 * g);
                    e[4 * g] = fmaf(-2.0f, __uint_as_float(v[4 * g]), w4.x);
                    e[4 * g + 1] = fmaf(-2.0f, __uint_as_float(v[4 * g + 1]), w4.y);
                    e[4 * g + 2] = fmaf(-2.0f, __uint_as_float(v[4 * g + 2]), w4.z);
                    e[4 * g + 3] = fmaf(-2.0f, __uint_as_float(v[4 * g + 3]), w4.w);
                }
                f32 lo[16];
#pragma unroll
                for (int h = 0; h < 16; ++h) lo[h] = fminf(e[h], e[h + 16]);
#pragma unroll
                for (int h = 0; h < 8; ++h) lo[h] = fminf(lo[h], lo[h + 8]);
#pragma unroll
                for (int h = 0; h < 4; ++h) lo[h] = fminf(lo[h], lo[h + 4]);
                const f32 emin = fminf(fminf(lo[0], lo[2]), fminf(lo[1], lo[3]));
                u32 m = 0;
                if (active && emin <= rq) {
#pragma unroll
                    for (int h = 0; h < 32; ++h) m |= u32(e[h] <= rq) << h;
                    const u32 cbase = j0 + u32(chunk * 32);
                    // +inf terms still pass while rq is +inf (list not yet full)
                    if (cbase + 32 > n) m &= cbase < n ? (1u << (n - cbase)) - 1u : 0u;
                    if (i >= cbase && i < cbase + 32) m &= ~(1u << (i - cbase));
                }
                mk[chunk] = m;
            }
            // (B) survivors. Few per tile, and at different lanes: they are
            // deferred into a per-thread buffer and evaluated in lockstep when
            // some lane's buffer would overflow (exact distance from the
            // L2-resident coordinates, then insertion). A tile with more
            // survivors than a buffer holds (the first tile of a block, while
            // the lists fill) is evaluated directly from the shared tile.
            const u32 tcnt = __popc(mk[0]) + __popc(mk[1]) + __popc(mk[2]) + __popc(mk[3]);
            if (__any_sync(0xffffffffu, tcnt != 0)) {
                if (__any_sync(0xffffffffu, tcnt > u32(TC_BUF))) {
                    flush();
                    bool changed = false;
#pragma unroll 1
                    for (int chunk = 0; chunk < TC_N / 32; ++chunk) {
#pragma unroll 1
                        for (u32 mm = mk[chunk]; mm; mm &= mm - 1) {
                            const u32 rr = u32(chunk * 32 + __ffs(mm) - 1);
                            f32 cb[TC_DIM];
                            swz_row(bt, rr, cb);
                            changed |= consider(j0 + rr, __fsqrt_rn(l2_sq_acc(RegVec<TC_DIM>{q}, RegVec<TC_DIM>{cb}, TC_DIM)));
                        }
                    }
                    if (changed) update_rq();
                } else {
                    if (__any_sync(0xffffffffu, nbuf + tcnt > u32(TC_BUF))) flush();
#pragma unroll 1
                    for (int chunk = 0; chunk < TC_N / 32; ++chunk)
                        for (u32 mm = mk[chunk]; mm; mm &= mm - 1)
                            S.buf[nbuf++][tid] = j0 + u32(chunk * 32 + __ffs(mm) - 1);
                }
            }
            ++uses_mma[sb];
            tc_fence_before();
            __syncthreads();   // TMEM buffer sb and shared stage sb are free again
            ++uses_b[st];
            if (tid == 0) {
                if (t + NSTAGE < ntiles) {
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    load_stage(st, t + NSTAGE);
                }
                S.stop = *((volatile u32*)err);   // one reader: the decision is block-uniform
            }
            __syncthreads();
            if (S.stop) {
                failed = true;
                break;
            }
        }
        flush();
        if (active) {
#pragma unroll
            for (int s = 0; s < TC_K; ++s)
                if (s < int(k)) {
                    ids[u64(i) * k + s] = lj[s];
                    if (dists) dists[u64(i) * k + s] = ld[s];
                }
        }
        __syncthreads();
    }
    if (exact_count && exact_evals) atomicAdd(exact_count, exact_evals);
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TC_N) : "memory");
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

bool knn_tc_applicable(u32 n, u32 dim, int kind, u32 k, const f32* x) {
    return kind == M_L2 && dim == u32(TC_DIM) && k >= 1 && k <= u32(TC_K) && n >= 2 &&
           (reinterpret_cast<uintptr_t>(x) & 15) == 0;
}

// Exact kNN lists through the tensor-core filter; returns the number of
// exact distance evaluations the filter let through.
u64 knn_tc(tt_ctx* c, const f32* x, u32 n, u32 k, u32* ids, f32* dists) {
    f32* nq = c->arena.get<f32>(S_MISC0, u64(n) + 1);
    // the norm terms are bulk-copied 128 per tile: pad to whole tiles
    const u64 wpad = (u64(n) + TC_N - 1) / TC_N * TC_N;
    f32* wc = c->arena.get<f32>(S_MISC3, wpad);
    u32* ctl = c->arena.get<u32>(S_MISC1, 4);   // [0] next block, [1] error word
    unsigned long long* cnt = c->arena.get<unsigned long long>(S_COUNT, 1);
    TT_CUDA(cudaMemsetAsync(ctl, 0, 4 * sizeof(u32), c->stream));
    TT_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), c->stream));
    k_norms<<<div_up(wpad, 256), 256, 0, c->stream>>>(x, n, u32(wpad), nq, wc);
    TT_LAUNCH("k_norms");
    CUtensorMap map;
    const cuuint64_t gdim[2] = {cuuint64_t(TC_DIM), cuuint64_t(n)};
    const cuuint64_t gstride[1] = {cuuint64_t(TC_DIM) * 4};
    const cuuint32_t box[2] = {cuuint32_t(TC_DIM), cuuint32_t(TC_M)};
    const cuuint32_t estride[2] = {1, 1};
    const CUresult r = encode_fn()(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<f32*>(x), gdim, gstride, box,
                                   estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw Error(TT_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string(int(r)) + ")");
    TT_CUDA(cudaFuncSetAttribute(k_knn_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, int(TC_SMEM)));
    const u32 nblocks = div_up(n, TC_M);
    const u32 grid = std::min<u32>(nblocks, 2 * u32(c->sms));
    k_knn_tc<<<grid, 128, TC_SMEM, c->stream>>>(map, x, n, k, nq, wc, ids, dists, ctl, ctl + 1, cnt);
    TT_LAUNCH("k_knn_tc");
    c->launches += 2;
    u32 e = 0;
    unsigned long long evals = 0;
    TT_CUDA(cudaMemcpyAsync(&e, ctl + 1, 4, cudaMemcpyDeviceToHost, c->stream));
    TT_CUDA(cudaMemcpyAsync(&evals, cnt, 8, cudaMemcpyDeviceToHost, c->stream));
    TT_CUDA(cudaStreamSynchronize(c->stream));
    if (e) throw Error(TT_ERR_TIMEOUT, "gb300: a bounded device wait timed out in the tensor-core kNN");
    return evals;
}

}  // namespace tt
