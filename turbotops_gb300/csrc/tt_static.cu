// tt_static.cu — tt_dense_distances_static: the distance matrix and the
// enclosing radius without any device allocation.
//
// Some callers cannot call cudaMalloc at the point where they need the
// distance matrix: host code that runs with all device memory already handed
// to its own pool (a framework that reserves the GPU's memory up front), or
// a latency-critical loop that must not take the device-wide synchronisation
// cudaMalloc/cudaFree imply. tt_dense_distances needs n + 1 words of scratch
// for the per-row maxima, which it takes from its context's arena; this
// variant takes them from a fixed array in the library's own device memory
// (g_rowmax below, kStaticRows + 1 words = 1 MiB per GPU that loads the
// library, held until the process exits). The caller passes the points and
// both outputs.
//
// Set-up: every call resolves the array's device address in the current
// context with cudaGetSymbolAddress (in host code the array's name is only a
// host-side stand-in, so kernels must be given that address); nothing is
// cached, so a device reset between calls is harmless. The first call on a
// device loads the library's module there: make it before any stream
// capture begins.
//
// Every call on a device shares the one array and leaves its last contents
// in it; the row maxima are cleared at the start of each call. Calls whose
// work overlaps on the GPU (different streams, no ordering between them)
// race on the array and must be serialised by the caller.

#include "tt_internal.cuh"

namespace tt {

constexpr u32 kStaticRows = 1u << 18;   // largest n accepted (a 256 GiB matrix)

static __device__ __align__(256) u32 g_rowmax[kStaticRows + 1];

void set_thread_error(const std::string& msg);   // tt_capi.cu

namespace {

__global__ void k_store_inf(f32* out) { *out = INFINITY; }

// Device address of g_rowmax in the current context, resolved on every call
// (a cheap lookup once the module is loaded): an address cached across calls
// would go stale if the caller reset the device or tore its context down.
u32* scratch_for() {
    void* p = nullptr;
    TT_CUDA(cudaGetSymbolAddress(&p, g_rowmax));
    return static_cast<u32*>(p);
}

}  // namespace
}  // namespace tt

using namespace tt;

extern "C" int tt_dense_distances_static(const float* x, uint32_t n, uint32_t dim, int kind, float p,
                                         float* mat, float* radius, void* stream) {
    try {
        if (kind < TT_METRIC_L1 || kind > TT_METRIC_LP) invalid("metric: unknown kind");
        if (kind == TT_METRIC_LP && !(p >= 1.0f)) invalid("metric: p must be in [1, inf]");
        if (n > kStaticRows)
            throw Error(TT_ERR_LENGTH, "gb300: tt_dense_distances_static accepts n <= 262144 points (its "
                                       "row-maximum scratch is a fixed 1 MiB device array)");
        if (!radius || (n && (!x || !mat))) invalid("gb300: null buffer");
        int device = 0;
        TT_CUDA(cudaGetDevice(&device));
        u32* rowmax = scratch_for();
        tt_ctx local;   // stream holder only: its arena is never touched here
        local.device = device;
        local.stream = static_cast<cudaStream_t>(stream);
        if (n == 0) {
            k_store_inf<<<1, 1, 0, local.stream>>>(radius);
            TT_LAUNCH("k_store_inf");
            return TT_OK;
        }
        // dense_matrix clears rowmax[0, n) before its kernel; min_bits
        // initialises its output word before folding the row maxima into it.
        dense_matrix(&local, x, n, dim, kind, p, mat, rowmax);
        min_bits(&local, rowmax, n, reinterpret_cast<u32*>(radius));
        return TT_OK;
    } catch (const Error& e) {
        set_thread_error(e.what());
        return e.status;
    } catch (const std::exception& e) {
        set_thread_error(e.what());
        return TT_ERR_INTERNAL;
    }
}
