// tt_dense.cu — full-layout distance matrix + enclosing radius.
//
// Replaces rips.hpp make_dense (:391-403, full layout) and
// DenseComplex::enclosing_radius (:370-380). One launch writes every entry of
// the n x n matrix (the diagonal evaluates to +0 exactly as the reference's
// zero-initialised diagonal) and folds each row's maximum into rowmax with an
// integer atomicMax on the float bits (monotone for non-negative floats).
// The enclosing radius is the minimum of the row maxima.
//
// Tiling: the 64 x 64 tiles on and above the diagonal (tt_dense_tile.cuh:
// each computed once, an off-diagonal tile written twice).
#include "tt_dense_tile.cuh"

namespace tt {

namespace {

constexpr int DN_T = 64;

template <int KIND, int DIM, bool VEC>
__global__ void __launch_bounds__(32 * dtile::kWarps)
k_dense(const f32* __restrict__ x, u32 n, u32 dim, f32 p, f32* __restrict__ mat, u32* __restrict__ rowmax) {
    if (blockIdx.y > blockIdx.x) return;   // below the diagonal: written by the mirror tile
    __shared__ dtile::Smem<DN_T> sm;
    dtile::sym_tile<KIND, DIM, VEC, DN_T>(x, n, dim, p, mat, rowmax, blockIdx.y * DN_T, blockIdx.x * DN_T, sm);
}

template <int KIND, int DIM>
void launch_dk(u32 n, cudaStream_t s, const f32* x, u32 dim, f32 p, f32* mat, u32* rowmax) {
    const u32 nb = div_up(n, DN_T);
    const dim3 grid(nb, nb);
    constexpr bool kVec = DIM > 0 && DIM % 4 == 0;   // rows of whole 16-byte groups
    if (kVec && (reinterpret_cast<uintptr_t>(x) & 15) == 0)
        k_dense<KIND, DIM, kVec><<<grid, 32 * dtile::kWarps, 0, s>>>(x, n, dim, p, mat, rowmax);
    else
        k_dense<KIND, DIM, false><<<grid, 32 * dtile::kWarps, 0, s>>>(x, n, dim, p, mat, rowmax);
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
