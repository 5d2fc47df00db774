// tt_dense_tile.cuh — one T x T tile of a full-layout distance matrix, shared
// by the single-cloud matrix (tt_dense.cu, make_dense) and the batched form
// (tt_batch.cu).
//
// Symmetry: d(i, j) and d(j, i) are the same bits ((a - b) and (b - a) differ
// only in sign), so a caller computes only the tiles on and above the
// diagonal, and an off-diagonal tile is written twice: directly, and
// transposed through shared memory, both times in whole row segments. That
// halves the distance arithmetic (a square root per entry for L2).
// A CTA of 8 warps: lane l holds the points of columns j0 + l + 32 c
// (c < T / 32) in registers (compile-time dimension) and warp w walks rows
// w, w + 8, ...: the lanes of a warp read the same row point (broadcast
// loads, 16 bytes at a time when VEC). Row maxima: the direct pass folds each
// column's maximum over the tile's rows (the rowmax of the column's point, by
// symmetry), the transposed pass each row's maximum over the tile's columns;
// one shared atomic a thread and one global atomic a row or column a tile. A
// tile on the diagonal covers both triangles of its block, so its column
// maxima are its row maxima.
#pragma once
#include "tt_internal.cuh"
#include "tt_metric.cuh"

namespace tt {
namespace dtile {

constexpr int kWarps = 8;

// The point of row i (DIM coordinates, 16-byte loads when VEC).
template <int DIM, bool VEC>
__device__ __forceinline__ void load_point(const f32* __restrict__ x, u64 i, f32 (&v)[DIM]) {
    if constexpr (VEC) {
        const float4* r = reinterpret_cast<const float4*>(x + i * DIM);
#pragma unroll
        for (int k = 0; k < DIM / 4; ++k) {
            const float4 t = __ldg(r + k);
            v[4 * k] = t.x, v[4 * k + 1] = t.y, v[4 * k + 2] = t.z, v[4 * k + 3] = t.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < DIM; ++k) v[k] = __ldg(x + i * DIM + k);
    }
}

template <int DIM>
struct Regs {
    const f32 (&v)[DIM];
    __device__ __forceinline__ f32 operator()(u32 k) const { return v[k]; }
};

template <int T>
struct Smem {
    f32 tile[T][T + 1];
    u32 cmax[T], rmax[T];
};

// The tile of rows i0.. and columns j0.. (i0 <= j0) of the n x n matrix mat
// of the points x; rowmax (nullable) gets the row maxima by atomicMax on the
// float bits. DIM > 0: the dimension at compile time; 0: any dimension, read
// from memory. Every thread of the CTA calls it; it synchronises the CTA
// and leaves the shared memory free again.
template <int KIND, int DIM, bool VEC, int T>
__device__ __forceinline__ void sym_tile(const f32* __restrict__ x, u32 n, u32 dim, f32 p, f32* __restrict__ mat,
                                         u32* __restrict__ rowmax, u32 i0, u32 j0, Smem<T>& sm) {
    static_assert(T % 32 == 0 && T <= 128, "tile edge: whole warps of columns");
    constexpr int CPT = T / 32;
    const bool diag = i0 == j0;
    const u32 lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x < T) sm.cmax[threadIdx.x] = sm.rmax[threadIdx.x] = 0u;
    __syncthreads();
    const u32 rows = min(u32(T), n - i0), cols = min(u32(T), n - j0);
    u32 cm[CPT];
#pragma unroll
    for (int c = 0; c < CPT; ++c) cm[c] = 0u;
    if constexpr (DIM > 0) {
        f32 xj[CPT][DIM];
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
            const u32 cc = lane + 32 * c;
            if (cc < cols) load_point<DIM, VEC>(x, j0 + cc, xj[c]);
            else {
#pragma unroll
                for (int k = 0; k < DIM; ++k) xj[c][k] = 0.0f;
            }
        }
#pragma unroll 2
        for (u32 r = w; r < rows; r += kWarps) {
            const u32 i = i0 + r;
            f32 xi[DIM];
            load_point<DIM, VEC>(x, i, xi);
            f32* row = mat + u64(i) * n + j0;
#pragma unroll
            for (int c = 0; c < CPT; ++c) {
                const u32 cc = lane + 32 * c;
                if (cc < cols) {
                    const f32 d = (i == j0 + cc) ? 0.0f : metric_dist(KIND, p, Regs<DIM>{xi}, Regs<DIM>{xj[c]}, DIM);
                    row[cc] = d;
                    sm.tile[r][cc] = d;
                    cm[c] = max(cm[c], __float_as_uint(d));
                }
            }
        }
    } else {
        for (u32 r = w; r < rows; r += kWarps) {
            const u32 i = i0 + r;
            f32* row = mat + u64(i) * n + j0;
#pragma unroll
            for (int c = 0; c < CPT; ++c) {
                const u32 cc = lane + 32 * c;
                if (cc < cols) {
                    const f32 d = (i == j0 + cc) ? 0.0f
                                                 : metric_dist(KIND, p, Row{x + u64(i) * dim},
                                                               Row{x + u64(j0 + cc) * dim}, dim);
                    row[cc] = d;
                    sm.tile[r][cc] = d;
                    cm[c] = max(cm[c], __float_as_uint(d));
                }
            }
        }
    }
#pragma unroll
    for (int c = 0; c < CPT; ++c)
        if (lane + 32 * c < cols) atomicMax(&sm.cmax[lane + 32 * c], cm[c]);
    __syncthreads();
    if (!diag) {
        // the transpose: entry (r, c) to (j0 + c, i0 + r), lanes along r
        u32 rm[CPT];
#pragma unroll
        for (int h = 0; h < CPT; ++h) rm[h] = 0u;
        for (u32 c = w; c < cols; c += kWarps) {
            f32* row = mat + u64(j0 + c) * n + i0;
#pragma unroll
            for (int h = 0; h < CPT; ++h) {
                const u32 r = lane + 32 * h;
                if (r < rows) {
                    const f32 d = sm.tile[r][c];
                    row[r] = d;
                    rm[h] = max(rm[h], __float_as_uint(d));
                }
            }
        }
#pragma unroll
        for (int h = 0; h < CPT; ++h)
            if (lane + 32 * h < rows) atomicMax(&sm.rmax[lane + 32 * h], rm[h]);
        __syncthreads();
    }
    if (rowmax && threadIdx.x < T) {
        if (threadIdx.x < cols) atomicMax(&rowmax[j0 + threadIdx.x], sm.cmax[threadIdx.x]);
        if (!diag && threadIdx.x < rows) atomicMax(&rowmax[i0 + threadIdx.x], sm.rmax[threadIdx.x]);
    }
    __syncthreads();   // the shared tile and maxima are free again
}

}  // namespace dtile
}  // namespace tt
