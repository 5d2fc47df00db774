// tt_sort.cu — device-wide primitives: exclusive scan, stream compaction and a
// stable LSD radix sort of 64-bit keys with an optional 32- or 64-bit payload.
//
// The filtration sorts (rips.hpp:775-839, redzed.hpp:545-613) are total
// orders on (diameter, index) and are reproduced exactly by sorting a packed
// 64-bit key, so ties never depend on sort stability or thread count.
//
// Radix sort: digits of up to 11 bits, 4096-key tiles (256 threads x 16
// keys). Per pass:
//   k_rs_upsweep   per-tile digit histogram -> hist[digit * tiles + tile]
//   scan           exclusive scan of hist (digit-major gives global offsets)
//   k_rs_scatter   stable in-tile ranking (warp match + per-warp counters,
//                  warp-major order), scatter to offsets
// Only the bits in which min key and max key differ are sorted (keys share
// every bit above the highest differing one), spread evenly over the fewest
// passes (25 bits: 9 + 8 + 8).
#include "tt_internal.cuh"

namespace tt {

namespace {

constexpr int RS_THREADS = 256, RS_ITEMS = 16, RS_TILE = RS_THREADS * RS_ITEMS;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_MAXBITS = 11, RS_BINS = 1 << RS_MAXBITS;   // digit width and bins per pass (at most)
constexpr int RS_LBITS = 8, RS_LBINS = 1 << RS_LBITS;       // the same for the local scatter (large inputs)
constexpr int SCAN_THREADS = 512, SCAN_ITEMS = 8, SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// ---------------------------------------------------------------------------
// Scan (exclusive, u64): tile sums, recursive scan of the sums, tile scan.
// ---------------------------------------------------------------------------
template <typename T>
__device__ T block_exclusive_scan(T v, T* warp_tot, T* total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    T inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) warp_tot[w] = inc;
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        T x = lane < nw ? warp_tot[lane] : T(0);
        T xi = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const T t = __shfl_up_sync(0xffffffffu, xi, o);
            if (lane >= o) xi += t;
        }
        if (lane < nw) warp_tot[lane] = xi - x;
        if (lane == nw - 1) *total = xi;
    }
    __syncthreads();
    const T r = inc - v + warp_tot[w];
    __syncthreads();
    return r;
}

template <typename T>
__global__ void k_tile_sums(const T* __restrict__ in, u64 n, T* __restrict__ sums) {
    pdl_wait();
    pdl_trigger();
    __shared__ T wt[32];
    __shared__ T tot;
    const u64 base = u64(blockIdx.x) * SCAN_TILE;
    T s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        const u64 k = base + u64(i) * SCAN_THREADS + threadIdx.x;
        if (k < n) s += in[k];
    }
    block_exclusive_scan<T>(s, wt, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

template <typename T>
__global__ void k_tile_scan(const T* __restrict__ in, u64 n, const T* __restrict__ offs,
                            T* __restrict__ out, T* __restrict__ total) {
    pdl_wait();
    pdl_trigger();
    __shared__ T wt[32];
    __shared__ T tot;
    const u64 base = u64(blockIdx.x) * SCAN_TILE + u64(threadIdx.x) * SCAN_ITEMS;
    T v[SCAN_ITEMS];
    T s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        v[i] = (base + i < n) ? in[base + i] : T(0);
        s += v[i];
    }
    T run = block_exclusive_scan<T>(s, wt, &tot) + (offs ? offs[blockIdx.x] : T(0));
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        if (base + i < n) out[base + i] = run;
        run += v[i];
    }
    if (total && blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) *total = run;
}

// ---------------------------------------------------------------------------
// Radix sort kernels.
// ---------------------------------------------------------------------------
// Which keys a tile (CTA b) holds and where its digit counts go. FlatTiles:
// the plain sort, tile b = keys [b RS_TILE, ...) of n (or of the count on the
// device), counts digit-major over the tiles. SegTiles: the segmented sort,
// tile b = keys [seg_off[s] + t RS_TILE, ...) of segment s (tiles never
// straddle segments), counts at hbase + digit * tcount + t, so that one
// exclusive scan of all segments' counts in order gives every key's final
// position (segment s's counts sum to its key count).
// kAllBins: the count layout reserves every bin of the widest digit for
// every tile (a segment's block of counts does not depend on the pass), so
// a pass with narrower digits writes zeros into the bins it does not use;
// the flat layout scans only the bins of the pass.
struct FlatTiles {
    static constexpr bool kAllBins = false;
    u64 n;
    const unsigned long long* ndev;
    u32 tiles;
    __device__ __forceinline__ bool valid(u32) const { return true; }
    __device__ __forceinline__ void range(u32 b, u64& lo, u64& hi) const {
        const u64 nn = ndev ? min(n, u64(*ndev)) : n;
        lo = u64(b) * RS_TILE;
        hi = lo < nn ? min(lo + RS_TILE, nn) : lo;
    }
    __device__ __forceinline__ u64 hidx(u32 b, u32 d) const { return u64(d) * tiles + b; }
};
struct SegTiles {
    static constexpr bool kAllBins = true;
    const SegTile* tl;
    const u64* seg_off;
    const u32* ntiles;   // tiles in the list (the grid covers its capacity)
    __device__ __forceinline__ bool valid(u32 b) const { return b < *ntiles; }
    __device__ __forceinline__ void range(u32 b, u64& lo, u64& hi) const {
        const SegTile e = tl[b];
        const u64 end = seg_off[e.seg + 1];
        lo = seg_off[e.seg] + u64(e.t) * RS_TILE;
        hi = lo < end ? min(lo + RS_TILE, end) : lo;
    }
    __device__ __forceinline__ u64 hidx(u32 b, u32 d) const {
        const SegTile e = tl[b];
        return e.hbase + u64(d) * e.tcount + e.t;
    }
};
// The lanes holding the same digit as this lane (a sentinel digit marks an
// empty slot). A warp whose 32 digits agree, the common case once the later
// passes see nearly sorted input, skips the match unit.
__device__ __forceinline__ u32 warp_peers(u32 dg) {
    if (__all_sync(0xffffffffu, dg == __shfl_sync(0xffffffffu, dg, 0))) return 0xffffffffu;
    return __match_any_sync(0xffffffffu, dg);
}

// Digits of up to RS_MAXBITS bits (a pass sorts `width` bits from `shift`).
// ndev (optional): the key count lives on the device (a graph-captured sort of
// a data-dependent number of keys, n the capacity); tiles past it are empty.
template <int BINS, typename TM>
__global__ void __launch_bounds__(RS_THREADS)
k_rs_upsweep(const u64* __restrict__ keys, TM tm, int shift, u32 width, u32* __restrict__ hist) {
    pdl_wait();
    pdl_trigger();
    __shared__ u32 h[RS_WARPS][BINS];
    if (!tm.valid(blockIdx.x)) return;   // past the list: no keys, no counts
    u64 tlo, n;   // this tile's keys: [tlo, n)
    tm.range(blockIdx.x, tlo, n);
    const u32 nd = 1u << width, mask = nd - 1u;
    for (u32 t = threadIdx.x; t < RS_WARPS * nd; t += RS_THREADS) h[t / nd][t % nd] = 0;
    __syncthreads();
    const int w = threadIdx.x >> 5;
    // Each thread counts RS_ITEMS consecutive keys, one shared atomic per run
    // of equal digits: nearly sorted input (the later passes) then costs one
    // atomic a thread instead of one a key on a single counter.
    const u64 base = tlo + u64(threadIdx.x) * RS_ITEMS;
    u64 kv[RS_ITEMS];
    const bool aligned = (reinterpret_cast<uintptr_t>(keys + base) & 15) == 0;
    if (base + RS_ITEMS <= n && aligned) {   // 16-byte loads
        const ulonglong2* p = reinterpret_cast<const ulonglong2*>(keys + base);
#pragma unroll
        for (int i = 0; i < RS_ITEMS / 2; ++i) {
            const ulonglong2 v = p[i];
            kv[2 * i] = v.x;
            kv[2 * i + 1] = v.y;
        }
    } else if (base + RS_ITEMS + 1 <= n && base > tlo) {
        // a run starting 8 bytes past a 16-byte boundary (a segment may
        // start anywhere): the aligned pairs from the key before it, which
        // belongs to the previous thread's run and is dropped
        const ulonglong2* p = reinterpret_cast<const ulonglong2*>(keys + base - 1);
        u64 prev = p[0].y;
#pragma unroll
        for (int i = 0; i < RS_ITEMS / 2; ++i) {
            const ulonglong2 v = p[i + 1];
            kv[2 * i] = prev;
            kv[2 * i + 1] = v.x;
            prev = v.y;
        }
    } else {
#pragma unroll
        for (int i = 0; i < RS_ITEMS; ++i) kv[i] = base + i < n ? keys[base + i] : 0ull;
    }
    const int cnt_valid = base >= n ? 0 : int(min(u64(RS_ITEMS), n - base));
    u32 cur = 0, run = 0;
#pragma unroll
    for (int i = 0; i < RS_ITEMS; ++i) {
        if (i < cnt_valid) {
            const u32 dg = u32(kv[i] >> shift) & mask;
            if (run && dg != cur) {
                atomicAdd(&h[w][cur], run);
                run = 0;
            }
            cur = dg;
            ++run;
        }
    }
    if (run) atomicAdd(&h[w][cur], run);
    __syncthreads();
    const u32 nb = TM::kAllBins ? u32(BINS) : nd;   // bins written (those past nd: zeros)
    for (u32 d = threadIdx.x; d < nb; d += RS_THREADS) {
        u32 s = 0;
        if (d < nd) {
#pragma unroll
            for (int q = 0; q < RS_WARPS; ++q) s += h[q][d];
        }
        hist[tm.hidx(blockIdx.x, d)] = s;
    }
}

template <typename V>
__global__ void __launch_bounds__(RS_THREADS)
k_rs_scatter(const u64* __restrict__ kin, u64* __restrict__ kout, const V* __restrict__ vin,
             V* __restrict__ vout, u64 n, const unsigned long long* __restrict__ ndev, int shift, u32 width,
             const u32* __restrict__ offs, u32 tiles) {
    pdl_wait();
    pdl_trigger();
    __shared__ u32 cnt[RS_WARPS][RS_BINS];   // per-warp running count, then warp prefix
    __shared__ u32 gbase[RS_BINS];
    if (ndev) n = min(n, u64(*ndev));
    if (u64(blockIdx.x) * RS_TILE >= n) return;
    const u32 nd = 1u << width, mask = nd - 1u;
    for (u32 t = threadIdx.x; t < RS_WARPS * nd; t += RS_THREADS) cnt[t / nd][t % nd] = 0;
    for (u32 d = threadIdx.x; d < nd; d += RS_THREADS) gbase[d] = offs[u64(d) * tiles + blockIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const u32 lt = (1u << lane) - 1u;
    // Warp w owns keys [base + w*32*ITEMS, base + (w+1)*32*ITEMS), item-major:
    // key (w, i, lane) precedes (w, i', lane') iff (i, lane) < (i', lane').
    const u64 base = u64(blockIdx.x) * RS_TILE + u64(w) * 32 * RS_ITEMS;
    u64 key[RS_ITEMS];
    u32 rank[RS_ITEMS];
#pragma unroll
    for (int i = 0; i < RS_ITEMS; ++i) {   // every load first, then the ranking
        const u64 k = base + u64(i) * 32 + lane;
        key[i] = k < n ? kin[k] : ~0ull;
    }
#pragma unroll
    for (int i = 0; i < RS_ITEMS; ++i) {
        const u64 k = base + u64(i) * 32 + lane;
        const bool ok = k < n;
        const u32 dg = ok ? u32(key[i] >> shift) & mask : RS_BINS;   // RS_BINS: no key
        const u32 peers = warp_peers(dg);
        const u32 before = __popc(peers & lt);
        const int leader = __ffs(peers) - 1;
        u32 prev = 0;
        if (lane == leader && dg < RS_BINS) {
            prev = cnt[w][dg];
            cnt[w][dg] = prev + __popc(peers);
        }
        prev = __shfl_sync(0xffffffffu, prev, leader);
        rank[i] = prev + before;
        __syncwarp();
    }
    __syncthreads();
    // exclusive prefix over warps, per digit
    for (u32 d = threadIdx.x; d < nd; d += RS_THREADS) {
        u32 s = 0;
#pragma unroll
        for (int q = 0; q < RS_WARPS; ++q) {
            const u32 c = cnt[q][d];
            cnt[q][d] = s;
            s += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < RS_ITEMS; ++i) {
        const u64 k = base + u64(i) * 32 + lane;
        if (k < n) {
            const u32 dg = u32(key[i] >> shift) & mask;
            const u32 pos = gbase[dg] + cnt[w][dg] + rank[i];
            kout[pos] = key[i];
            if (vin) vout[pos] = vin[k];
        }
    }
}

// The same pass for large inputs, digits of at most RS_LBITS bits: the tile
// is first ordered by digit in shared memory (stable), then written out in
// that order, so the keys of one digit leave a tile as one contiguous run
// (about RS_TILE / 2^width keys) instead of scattered 8-byte writes.
template <typename V, bool VALS, typename TM>
__global__ void __launch_bounds__(RS_THREADS)
k_rs_scatter_local(const u64* __restrict__ kin, u64* __restrict__ kout, const V* __restrict__ vin,
                   V* __restrict__ vout, TM tm, int shift, u32 width, const u32* __restrict__ offs) {
    pdl_wait();
    pdl_trigger();
    __shared__ u64 skey[RS_TILE];
    __shared__ V sval[VALS ? RS_TILE : 1];
    __shared__ u32 cnt[RS_WARPS][RS_LBINS];   // per-warp running count, then warp prefix
    __shared__ u32 gbase[RS_LBINS];
    __shared__ u32 tstart[RS_LBINS];          // the digit's first position in the ordered tile
    __shared__ u32 wsum[RS_WARPS];
    __shared__ u32 mbins[RS_WARPS][RS_LBINS]; // per-warp lane masks by digit (the ranking below)
    if (!tm.valid(blockIdx.x)) return;
    u64 tbase, n;   // this tile's keys: [tbase, n)
    tm.range(blockIdx.x, tbase, n);
    if (tbase >= n) return;
    const u32 nd = 1u << width, mask = nd - 1u;
    for (u32 t = threadIdx.x; t < RS_WARPS * RS_LBINS; t += RS_THREADS) {
        cnt[t / RS_LBINS][t % RS_LBINS] = 0;
        mbins[t / RS_LBINS][t % RS_LBINS] = 0;
    }
    for (u32 d = threadIdx.x; d < nd; d += RS_THREADS) gbase[d] = offs[tm.hidx(blockIdx.x, d)];
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const u32 lt = (1u << lane) - 1u;
    // ranks within the warp's keys, item-major (as k_rs_scatter)
    const u64 base = tbase + u64(w) * 32 * RS_ITEMS;
    u64 key[RS_ITEMS];
    V val[VALS ? RS_ITEMS : 1];
    u32 rank[RS_ITEMS];
    // every load first (all in flight at once), then the ranking
#pragma unroll
    for (int i = 0; i < RS_ITEMS; ++i) {
        const u64 k = base + u64(i) * 32 + lane;
        const bool ok = k < n;
        key[i] = ok ? kin[k] : ~0ull;
        if constexpr (VALS) val[i] = ok ? vin[k] : V(0);
    }
#pragma unroll
    for (int i = 0; i < RS_ITEMS; ++i) {
        const u64 k = base + u64(i) * 32 + lane;
        const bool ok = k < n;
        const u32 dg = ok ? u32(key[i] >> shift) & mask : u32(RS_LBINS);   // RS_LBINS: no key
        // lanes of one digit: each sets its bit in the warp's mask for the digit
        // (a shared atomic, instead of the match unit), all read the mask back,
        // and the lowest of them clears it before the next item
        const bool has = dg < u32(RS_LBINS);
        u32 peers;
        if (__all_sync(0xffffffffu, dg == __shfl_sync(0xffffffffu, dg, 0))) {   // one digit (warp-uniform branch)
            peers = has ? 0xffffffffu : 0u;
        } else {
            if (has) atomicOr(&mbins[w][dg], 1u << lane);
            __syncwarp();
            peers = has ? mbins[w][dg] : 0u;
            __syncwarp();
            if (has && lane == u32(__ffs(peers) - 1)) mbins[w][dg] = 0u;
            __syncwarp();
        }
        const u32 before = __popc(peers & lt);
        const int leader = __ffs(peers) - 1;
        u32 prev = 0;
        if (lane == leader && dg < u32(RS_LBINS)) {
            prev = cnt[w][dg];
            cnt[w][dg] = prev + __popc(peers);
        }
        prev = __shfl_sync(0xffffffffu, prev, leader);
        rank[i] = prev + before;
        __syncwarp();
    }
    __syncthreads();
    // per digit: exclusive prefix over warps and the digit's total; then an
    // exclusive scan of the totals over the digits (one digit a thread)
    u32 tot = 0;
    const u32 d = threadIdx.x;   // RS_LBINS == RS_THREADS
    if (d < nd) {
#pragma unroll
        for (int q = 0; q < RS_WARPS; ++q) {
            const u32 c = cnt[q][d];
            cnt[q][d] = tot;
            tot += c;
        }
    }
    u32 inc = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const u32 y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    u32 wpre = 0;
#pragma unroll
    for (int q = 0; q < RS_WARPS; ++q) wpre += q < w ? wsum[q] : 0u;
    tstart[d] = wpre + inc - tot;
    __syncthreads();
    // order the tile by digit in shared memory
#pragma unroll
    for (int i = 0; i < RS_ITEMS; ++i) {
        const u64 k = base + u64(i) * 32 + lane;
        if (k < n) {
            const u32 dg = u32(key[i] >> shift) & mask;
            const u32 lp = tstart[dg] + cnt[w][dg] + rank[i];
            skey[lp] = key[i];
            if constexpr (VALS) sval[lp] = val[i];
        }
    }
    __syncthreads();
    // write out in that order: runs of one digit go to consecutive positions
    const u32 valid = u32(min(u64(RS_TILE), n - tbase));
    for (u32 j = threadIdx.x; j < valid; j += RS_THREADS) {
        const u64 kk = skey[j];
        const u32 dg = u32(kk >> shift) & mask;
        const u32 pos = gbase[dg] + (j - tstart[dg]);
        kout[pos] = kk;
        if constexpr (VALS) vout[pos] = sval[j];
    }
}
static_assert(RS_LBINS == RS_THREADS, "one digit a thread in the local scatter's scan");
static_assert(RS_TILE == int(kSegTileKeys), "the segmented sort's tiles are the radix tiles");

__global__ void k_minmax(const u64* __restrict__ keys, u64 n, unsigned long long* __restrict__ mm) {
    u64 lo = ~0ull, hi = 0;
    for (u64 i = u64(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += u64(gridDim.x) * blockDim.x) {
        const u64 k = keys[i];
        lo = min(lo, k);
        hi = max(hi, k);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        lo = min(lo, (u64)__shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, (u64)__shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&mm[0], (unsigned long long)lo);
        atomicMax(&mm[1], (unsigned long long)hi);
    }
}

}  // namespace

template <typename T>
void scan_exclusive(tt_ctx* c, const T* in, T* out, u64 n, T* total, int depth) {
    if (n == 0) {
        if (total) TT_CUDA(cudaMemsetAsync(total, 0, sizeof(T), c->stream));
        return;
    }
    const u64 tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (tiles == 1) {
        launch_pdl(k_tile_scan<T>, 1, SCAN_THREADS, 0, c->stream, in, n, static_cast<const T*>(nullptr), out, total);
        TT_LAUNCH("k_tile_scan");
        c->launches += 1;
        return;
    }
    if (depth > 2) invalid("scan: input too large");
    // sums[0..tiles) tile totals, sums[tiles..2 tiles) their exclusive scan;
    // each recursion level has its own scratch slot
    T* sums = c->arena.get<T>(depth == 0 ? S_SCAN : depth == 1 ? S_SCAN2 : S_SCAN3, 2 * tiles + 2);
    launch_pdl(k_tile_sums<T>, u32(tiles), SCAN_THREADS, 0, c->stream, in, n, sums);
    TT_LAUNCH("k_tile_sums");
    if (tiles <= SCAN_TILE) {
        launch_pdl(k_tile_scan<T>, 1, SCAN_THREADS, 0, c->stream, static_cast<const T*>(sums), tiles,
                   static_cast<const T*>(nullptr), sums + tiles, static_cast<T*>(nullptr));
        TT_LAUNCH("k_tile_scan");
        c->launches += 1;
    } else {
        scan_exclusive<T>(c, sums, sums + tiles, tiles, nullptr, depth + 1);
    }
    launch_pdl(k_tile_scan<T>, u32(tiles), SCAN_THREADS, 0, c->stream, in, n, static_cast<const T*>(sums + tiles), out,
               total);
    TT_LAUNCH("k_tile_scan");
    c->launches += 2;
}

template void scan_exclusive<u64>(tt_ctx*, const u64*, u64*, u64, u64*, int);
template void scan_exclusive<u32>(tt_ctx*, const u32*, u32*, u64, u32*, int);

// Sorts keys[0..n) ascending (stable, with the optional payload). Returns the
// buffers that hold the result: the caller's (keys, vals) or the arena
// scratch (kbuf, vbuf) — 'swapped' tells which.
template <typename V>
bool radix_sort(tt_ctx* c, u64* keys, V* vals, u64 n, u64* kbuf, V* vbuf, int force_bits, int lo_bit,
                const unsigned long long* ndev) {
    if (n <= 1) return false;
    int bits = force_bits;
    if (bits <= 0) {
        unsigned long long* mm = c->arena.get<unsigned long long>(S_MISC3, 2);
        const unsigned long long init[2] = {~0ull, 0ull};
        TT_CUDA(cudaMemcpyAsync(mm, init, sizeof(init), cudaMemcpyHostToDevice, c->stream));
        k_minmax<<<std::min<u32>(div_up(n, 256), 8 * kSMs), 256, 0, c->stream>>>(keys, n, mm);
        TT_LAUNCH("k_minmax");
        ++c->launches;
        unsigned long long h[2];
        TT_CUDA(cudaMemcpyAsync(h, mm, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
        TT_CUDA(cudaStreamSynchronize(c->stream));
        const u64 diff = (h[0] ^ h[1]) >> lo_bit;
        bits = diff ? 64 - __builtin_clzll(diff) : 0;
    }
    const u32 tiles = div_up(n, RS_TILE);
    u32* hist = c->arena.get<u32>(S_SORT_HIST, u64(tiles) * RS_BINS + 1);
    u64 *ka = keys, *kb = kbuf;
    V *va = vals, *vb = vbuf;
    bool swapped = false;
    // as few passes as digits of up to RS_MAXBITS bits allow, the bits
    // spread evenly over them (25 bits: 9 + 8 + 8; 11 bits: one pass). Inputs
    // far beyond L2 take digits of at most RS_LBITS bits and the local
    // scatter: more passes, each writing contiguous runs.
    const bool local = n >= (u64(1) << 22);
    const int maxbits = local ? RS_LBITS : RS_MAXBITS;
    const int passes = (bits + maxbits - 1) / maxbits;
    int shift = lo_bit;
    for (int q = 0; q < passes; ++q) {
        const int width = (lo_bit + bits - shift + (passes - q) - 1) / (passes - q);
        const FlatTiles tm{n, ndev, tiles};
        if (local)
            launch_pdl(k_rs_upsweep<RS_LBINS, FlatTiles>, tiles, RS_THREADS, 0, c->stream, static_cast<const u64*>(ka), tm, shift,
                       u32(width), hist);
        else
            launch_pdl(k_rs_upsweep<RS_BINS, FlatTiles>, tiles, RS_THREADS, 0, c->stream, static_cast<const u64*>(ka), tm, shift,
                       u32(width), hist);
        TT_LAUNCH("k_rs_upsweep");
        scan_exclusive<u32>(c, hist, hist, u64(tiles) << width, nullptr, 0);
        if (local && va)
            launch_pdl(k_rs_scatter_local<V, true, FlatTiles>, tiles, RS_THREADS, 0, c->stream,
                       static_cast<const u64*>(ka), kb, static_cast<const V*>(va), vb, tm, shift, u32(width),
                       static_cast<const u32*>(hist));
        else if (local)
            launch_pdl(k_rs_scatter_local<V, false, FlatTiles>, tiles, RS_THREADS, 0, c->stream,
                       static_cast<const u64*>(ka), kb, static_cast<const V*>(va), vb, tm, shift, u32(width),
                       static_cast<const u32*>(hist));
        else
            launch_pdl(k_rs_scatter<V>, tiles, RS_THREADS, 0, c->stream, static_cast<const u64*>(ka), kb,
                       static_cast<const V*>(va), vb, n, ndev, shift, u32(width), static_cast<const u32*>(hist), tiles);
        TT_LAUNCH("k_rs_scatter");
        c->launches += 2;
        std::swap(ka, kb);
        std::swap(va, vb);
        swapped = !swapped;
        shift += width;
    }
    return swapped;
}

template bool radix_sort<u32>(tt_ctx*, u64*, u32*, u64, u64*, u32*, int, int, const unsigned long long*);
template bool radix_sort<u64>(tt_ctx*, u64*, u64*, u64, u64*, u64*, int, int, const unsigned long long*);

// Each segment [seg_off[s], seg_off[s + 1]) sorted on its own (stable) by key
// bits [lo_bit, lo_bit + bits): the keys never leave their segment, so bits
// that only tell segments apart need no pass. 8-bit digits and the local
// scatter (runs of one digit leave a tile together); the tiles and their
// count offsets come from the caller (SegTile), the segment bounds from the
// device. The list's length is on the device (ntiles_dev); max_tiles and
// hist_entries bound it and its counts (the grids and the scan cover them:
// counts past the list's only shift prefixes past its keys). Returns whether
// the result is in kbuf.
bool radix_sort_segments(tt_ctx* c, u64* keys, u64* kbuf, const u64* seg_off, const SegTile* tl,
                         const u32* ntiles_dev, u32 max_tiles, u64 hist_entries, int bits, int lo_bit) {
    const u32 ntiles = max_tiles;
    if (ntiles == 0 || bits <= 0) return false;
    u32* hist = c->arena.get<u32>(S_SORT_HIST, hist_entries + 1);
    u64 *ka = keys, *kb = kbuf;
    bool swapped = false;
    const int passes = (bits + RS_LBITS - 1) / RS_LBITS;
    int shift = lo_bit;
    const SegTiles tm{tl, seg_off, ntiles_dev};
    for (int q = 0; q < passes; ++q) {
        const int width = (lo_bit + bits - shift + (passes - q) - 1) / (passes - q);
        launch_pdl(k_rs_upsweep<RS_LBINS, SegTiles>, ntiles, RS_THREADS, 0, c->stream, static_cast<const u64*>(ka), tm, shift,
                   u32(width), hist);
        TT_LAUNCH("k_rs_upsweep");
        scan_exclusive<u32>(c, hist, hist, hist_entries, nullptr, 0);
        launch_pdl(k_rs_scatter_local<u32, false, SegTiles>, ntiles, RS_THREADS, 0, c->stream,
                   static_cast<const u64*>(ka), kb, static_cast<const u32*>(nullptr), static_cast<u32*>(nullptr), tm,
                   shift, u32(width), static_cast<const u32*>(hist));
        TT_LAUNCH("k_rs_scatter");
        c->launches += 2;
        std::swap(ka, kb);
        swapped = !swapped;
        shift += width;
    }
    return swapped;
}

// Sort keys in place (result always back in `keys`, payload in `vals`).
template <typename V>
void radix_sort_inplace(tt_ctx* c, u64* keys, V* vals, u64 n, int force_bits) {
    if (n <= 1) return;
    u64* kb = c->arena.get<u64>(S_SORT_A, n);
    V* vb = vals ? c->arena.get<V>(S_SORT_VA, n) : nullptr;
    if (radix_sort<V>(c, keys, vals, n, kb, vb, force_bits)) {
        TT_CUDA(cudaMemcpyAsync(keys, kb, n * sizeof(u64), cudaMemcpyDeviceToDevice, c->stream));
        if (vals) TT_CUDA(cudaMemcpyAsync(vals, vb, n * sizeof(V), cudaMemcpyDeviceToDevice, c->stream));
    }
}

// Every scratch slot radix_sort of n keys may grow (for callers that record
// their work into a CUDA graph, where no allocation may happen).
void radix_reserve(tt_ctx* c, u64 n) { radix_reserve_entries(c, div_up(n, RS_TILE) * RS_BINS); }

void radix_reserve_entries(tt_ctx* c, u64 entries) {
    c->arena.get<u32>(S_SORT_HIST, entries + 1);
    u64 e = entries;   // histogram entries, scanned level by level
    const int slots[3] = {S_SCAN, S_SCAN2, S_SCAN3};
    for (int d = 0; d < 3 && e > u64(SCAN_TILE); ++d) {
        const u64 t = (e + SCAN_TILE - 1) / SCAN_TILE;
        c->arena.get<u32>(slots[d], 2 * t + 2);
        e = t;
    }
}

template void radix_sort_inplace<u32>(tt_ctx*, u64*, u32*, u64, int);
template void radix_sort_inplace<u64>(tt_ctx*, u64*, u64*, u64, int);

}  // namespace tt
