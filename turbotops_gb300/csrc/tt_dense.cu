// tt_dense.cu — full-layout distance matrix + enclosing radius.
//
// Replaces rips.hpp make_dense (:391-403, full layout) and
// DenseComplex::enclosing_radius (:370-380). One launch writes every entry of
// the n x n matrix (the diagonal evaluates to +0 exactly as the reference's
// zero-initialised diagonal) and folds each row's maximum into rowmax with an
// integer atomicMax on the float bits (monotone for non-negative floats).
// The enclosing radius is the minimum of the row maxima.
//
// Tiling: a CTA owns a 32-row x 64-column tile; the tile's points are staged
// in shared memory (dim <= kSmemDim) so each point row is read from HBM/L2
// once per tile; consecutive threads write consecutive columns (coalesced,
// 256-byte row segments).
#include "tt_internal.cuh"
#include "tt_metric.cuh"

namespace tt {

namespace {

constexpr int TR = 32, TC = 64, TY = 4;
constexpr u32 kSmemDim = 64;

template <int KIND>
__global__ void __launch_bounds__(TC* TY)
k_dense(const f32* __restrict__ x, u32 n, u32 dim, f32 p, f32* __restrict__ mat,
        u32* __restrict__ rowmax) {
    extern __shared__ f32 sm[];
    const u32 i0 = blockIdx.y * TR, j0 = blockIdx.x * TC;
    const u32 tx = threadIdx.x, ty = threadIdx.y, tid = ty * TC + tx;
    const bool staged = dim <= kSmemDim;
    const u32 ld = dim + 1;   // padded row stride (odd for dim even: fewer bank conflicts)
    f32* Xi = sm;
    f32* Xj = sm + TR * ld;
    if (staged) {
        for (u32 t = tid; t < TR * dim; t += TC * TY) {
            const u32 r = t / dim, k = t - r * dim;
            Xi[r * ld + k] = (i0 + r < n) ? x[u64(i0 + r) * dim + k] : 0.0f;
        }
        for (u32 t = tid; t < TC * dim; t += TC * TY) {
            const u32 r = t / dim, k = t - r * dim;
            Xj[r * ld + k] = (j0 + r < n) ? x[u64(j0 + r) * dim + k] : 0.0f;
        }
        __syncthreads();
    }
    __shared__ u32 smax[TR];
    if (tid < TR) smax[tid] = 0u;
    __syncthreads();
    const u32 j = j0 + tx;
    for (u32 r = ty; r < TR; r += TY) {
        const u32 i = i0 + r;
        if (i >= n) break;
        f32 d = 0.0f;
        if (j < n) {
            const f32* a = staged ? Xi + r * ld : x + u64(i) * dim;
            const f32* b = staged ? Xj + tx * ld : x + u64(j) * dim;
            d = (i == j) ? 0.0f : metric_dist(KIND, p, Row{a}, Row{b}, dim);
            mat[u64(i) * n + j] = d;
        }
        if (rowmax) {
            // warp max over the 32 columns this warp holds, one smem atomic
            u32 v = __float_as_uint(d);
#pragma unroll
            for (int o = 16; o; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
            if ((tx & 31) == 0) atomicMax(&smax[r], v);
        }
    }
    if (rowmax) {
        __syncthreads();
        if (tid < TR && i0 + tid < n) atomicMax(&rowmax[i0 + tid], smax[tid]);
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
    const dim3 grid(div_up(n, TC), div_up(n, TR)), block(TC, TY);
    const size_t smem = dim <= kSmemDim ? sizeof(f32) * (TR + TC) * (dim + 1) : 0;
    switch (kind) {
        case M_L1: k_dense<M_L1><<<grid, block, smem, c->stream>>>(x, n, dim, p, mat, rowmax); break;
        case M_L2: k_dense<M_L2><<<grid, block, smem, c->stream>>>(x, n, dim, p, mat, rowmax); break;
        case M_LINF: k_dense<M_LINF><<<grid, block, smem, c->stream>>>(x, n, dim, p, mat, rowmax); break;
        default: k_dense<M_LP><<<grid, block, smem, c->stream>>>(x, n, dim, p, mat, rowmax); break;
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
