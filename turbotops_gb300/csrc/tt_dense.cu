// tt_dense.cu — full-layout distance matrix + enclosing radius.
//
// Replaces rips.hpp make_dense (:391-403, full layout) and
// DenseComplex::enclosing_radius (:370-380). One launch writes every entry of
// the n x n matrix (the diagonal evaluates to +0 exactly as the reference's
// zero-initialised diagonal) and folds each row's maximum into rowmax with an
// integer atomicMax on the float bits (monotone for non-negative floats).
// The enclosing radius is the minimum of the row maxima.
//
// Symmetry: d(i, j) and d(j, i) are the same bits ((a - b) and (b - a) differ
// only in sign), so only the tiles on and above the diagonal are computed,
// and an off-diagonal tile is written twice: directly, and transposed through
// shared memory, both times in 256-byte row segments. That halves the
// distance arithmetic (a square root per entry for L2), which bounded the
// all-entries form on instruction issue.
// Tiling: a CTA of 8 warps owns a 64 x 64 tile (rows i0.., columns j0..,
// i0 <= j0). Lane l of every warp holds the points of columns j0 + l and
// j0 + l + 32 in registers (compile-time dimension) and warp w walks rows w,
// w + 8, ...: the lanes of a warp read the same row point (broadcast loads,
// 16 bytes at a time when the rows allow). Row maxima: the direct pass folds
// each column's maximum over the tile's rows (rowmax of the column's point,
// by symmetry), the transposed pass each row's maximum over the tile's
// columns; one shared atomic a thread and one global atomic a row or column
// a tile, no cross-lane reduction per entry. A tile on the diagonal covers
// both triangles of its block, so its column maxima are its row maxima.
#include "tt_internal.cuh"
#include "tt_metric.cuh"

namespace tt {

namespace {

constexpr int DN_T = 64, DN_WARPS = 8;

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

// DIM > 0: the dimension at compile time; 0: any dimension, read from memory.
template <int KIND, int DIM, bool VEC>
__global__ void __launch_bounds__(32 * DN_WARPS)
k_dense(const f32* __restrict__ x, u32 n, u32 dim, f32 p, f32* __restrict__ mat, u32* __restrict__ rowmax) {
    if (blockIdx.y > blockIdx.x) return;   // below the diagonal: written by the mirror tile
    __shared__ f32 tile[DN_T][DN_T + 1];
    __shared__ u32 cmax[DN_T], rmax[DN_T];
    const u32 i0 = blockIdx.y * DN_T, j0 = blockIdx.x * DN_T;
    const bool diag = i0 == j0;
    const u32 lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x < DN_T) cmax[threadIdx.x] = rmax[threadIdx.x] = 0u;
    __syncthreads();
    const u32 rows = min(u32(DN_T), n - i0), cols = min(u32(DN_T), n - j0);
    u32 cm[2] = {0u, 0u};
    if constexpr (DIM > 0) {
        f32 xj[2][DIM];
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const u32 cc = lane + 32 * c;
            if (cc < cols) load_point<DIM, VEC>(x, j0 + cc, xj[c]);
            else {
#pragma unroll
                for (int k = 0; k < DIM; ++k) xj[c][k] = 0.0f;
            }
        }
#pragma unroll 2
        for (u32 r = w; r < rows; r += DN_WARPS) {
            const u32 i = i0 + r;
            f32 xi[DIM];
            load_point<DIM, VEC>(x, i, xi);
            f32* row = mat + u64(i) * n + j0;
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const u32 cc = lane + 32 * c;
                if (cc < cols) {
                    const f32 d = (i == j0 + cc) ? 0.0f : metric_dist(KIND, p, Regs<DIM>{xi}, Regs<DIM>{xj[c]}, DIM);
                    row[cc] = d;
                    tile[r][cc] = d;
                    cm[c] = max(cm[c], __float_as_uint(d));
                }
            }
        }
    } else {
        for (u32 r = w; r < rows; r += DN_WARPS) {
            const u32 i = i0 + r;
            f32* row = mat + u64(i) * n + j0;
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const u32 cc = lane + 32 * c;
                if (cc < cols) {
                    const f32 d = (i == j0 + cc) ? 0.0f
                                                 : metric_dist(KIND, p, Row{x + u64(i) * dim},
                                                               Row{x + u64(j0 + cc) * dim}, dim);
                    row[cc] = d;
                    tile[r][cc] = d;
                    cm[c] = max(cm[c], __float_as_uint(d));
                }
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 2; ++c)
        if (lane + 32 * c < cols) atomicMax(&cmax[lane + 32 * c], cm[c]);
    __syncthreads();
    if (!diag) {
        // the transpose: entry (r, c) to (j0 + c, i0 + r), lanes along r
        u32 rm[2] = {0u, 0u};
        for (u32 c = w; c < cols; c += DN_WARPS) {
            f32* row = mat + u64(j0 + c) * n + i0;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const u32 r = lane + 32 * h;
                if (r < rows) {
                    const f32 d = tile[r][c];
                    row[r] = d;
                    rm[h] = max(rm[h], __float_as_uint(d));
                }
            }
        }
#pragma unroll
        for (int h = 0; h < 2; ++h)
            if (lane + 32 * h < rows) atomicMax(&rmax[lane + 32 * h], rm[h]);
        __syncthreads();
    }
    if (rowmax && threadIdx.x < DN_T) {
        if (threadIdx.x < cols) atomicMax(&rowmax[j0 + threadIdx.x], cmax[threadIdx.x]);
        if (!diag && threadIdx.x < rows) atomicMax(&rowmax[i0 + threadIdx.x], rmax[threadIdx.x]);
    }
}

template <int KIND, int DIM>
void launch_dk(u32 n, cudaStream_t s, const f32* x, u32 dim, f32 p, f32* mat, u32* rowmax) {
    const u32 nb = div_up(n, DN_T);
    const dim3 grid(nb, nb);
    constexpr bool kVec = DIM > 0 && DIM % 4 == 0;   // rows of whole 16-byte groups
    if (kVec && (reinterpret_cast<uintptr_t>(x) & 15) == 0)
        k_dense<KIND, DIM, kVec><<<grid, 32 * DN_WARPS, 0, s>>>(x, n, dim, p, mat, rowmax);
    else
        k_dense<KIND, DIM, false><<<grid, 32 * DN_WARPS, 0, s>>>(x, n, dim, p, mat, rowmax);
}

// (Lp indexes the coordinates at run time: above four dimensions its register
// copies would live in local memory, so it reads rows instead.)
template <int KIND>
void launch_dense(u32 n, cudaStream_t s, const f32* x, u32 dim, f32 p, f32* mat, u32* rowmax) {
    if constexpr (KIND == M_LP) {
        switch (dim) {
            case 2: launch_dk<KIND, 2>(n, s, x, dim, p, mat, rowmax); break;
            case 3: launch_dk<KIND, 3>(n, s, x, dim, p, mat, rowmax); break;
            case 4: launch_dk<KIND, 4>(n, s, x, dim, p, mat, rowmax); break;
            default: launch_dk<KIND, 0>(n, s, x, dim, p, mat, rowmax); break;
        }
    } else {
        switch (dim) {
            case 2: launch_dk<KIND, 2>(n, s, x, dim, p, mat, rowmax); break;
            case 3: launch_dk<KIND, 3>(n, s, x, dim, p, mat, rowmax); break;
            case 4: launch_dk<KIND, 4>(n, s, x, dim, p, mat, rowmax); break;
            case 8: launch_dk<KIND, 8>(n, s, x, dim, p, mat, rowmax); break;
            case 16: launch_dk<KIND, 16>(n, s, x, dim, p, mat, rowmax); break;
            case 32: launch_dk<KIND, 32>(n, s, x, dim, p, mat, rowmax); break;
            default: launch_dk<KIND, 0>(n, s, x, dim, p, mat, rowmax); break;
        }
    }
}

__global__ void k_min_bits(const u32* __restrict__ v, u32 n, u32* __restrict__ out) {
    u32 m = 0xffffffffu;
    for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) m = min(m, v[i]);
#pragma unroll
    for (int o = 16; o; o >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMin(out, m);
}

}  // namespace

void dense_matrix(tt_ctx* c, const f32* x, u32 n, u32 dim, int kind, f32 p, f32* mat,
                  u32* rowmax) {
    if (n == 0) return;
    if (rowmax) TT_CUDA(cudaMemsetAsync(rowmax, 0, sizeof(u32) * n, c->stream));
    switch (kind) {
        case M_L1: launch_dense<M_L1>(n, c->stream, x, dim, p, mat, rowmax); break;
        case M_L2: launch_dense<M_L2>(n, c->stream, x, dim, p, mat, rowmax); break;
        case M_LINF: launch_dense<M_LINF>(n, c->stream, x, dim, p, mat, rowmax); break;
        default: launch_dense<M_LP>(n, c->stream, x, dim, p, mat, rowmax); break;
    }
    TT_LAUNCH("k_dense");
    ++c->launches;
}

void min_bits(tt_ctx* c, const u32* v, u32 n, u32* out) {
    TT_CUDA(cudaMemsetAsync(out, 0xff, sizeof(u32), c->stream));
    if (n == 0) return;
    k_min_bits<<<std::min<u32>(div_up(n, 256), 4 * kSMs), 256, 0, c->stream>>>(v, n, out);
    TT_LAUNCH("k_min_bits");
    ++c->launches;
}

}  // namespace tt
