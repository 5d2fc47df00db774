// tt_common.cuh — shared definitions of the GB300 front-end library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/turbotops_gb300.h"

namespace tt {

using u8 = uint8_t;
using u16 = uint16_t;
using u32 = uint32_t;
using u64 = uint64_t;
using i64 = int64_t;
using f32 = float;

constexpr int kSMs = 152;          // GB300: 2 dies x 76 SMs
constexpr u64 kNone = ~0ull;

// Errors thrown inside the library and mapped to TT_* status codes at the
// C-ABI boundary (tt_capi.cu). The message is the reference's message where
// the reference has one for the same condition.
struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess)
        throw Error(TT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define TT_CUDA(x) ::tt::check((x), #x)
#define TT_LAUNCH(what) ::tt::check(cudaGetLastError(), what)

inline void invalid(const std::string& m) { throw Error(TT_ERR_INVALID, m); }

inline u32 div_up(u64 a, u64 b) { return u32((a + b - 1) / b); }

__host__ __device__ inline u32 fbits(f32 d) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(d);
#else
    u32 u;
    __builtin_memcpy(&u, &d, 4);
    return u;
#endif
}
__host__ __device__ inline f32 bitsf(u32 u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    f32 d;
    __builtin_memcpy(&d, &u, 4);
    return d;
#endif
}

// Device-memory arena owned by a context: one cudaMalloc'd slab per size
// class, reused across calls, so steady-state calls allocate nothing.
struct Arena {
    struct Slab {
        void* p = nullptr;
        size_t bytes = 0;
    };
    std::vector<Slab> slabs;   // indexed by slot
    // Host-side fault injection (tt_ctx_inject_alloc_failure): the
    // fail_in-th next slab allocation reports cudaErrorMemoryAllocation
    // without calling cudaMalloc. 0 = off.
    unsigned fail_in = 0;
    void* get(int slot, size_t bytes) {
        if (slot >= int(slabs.size())) slabs.resize(slot + 1);
        Slab& s = slabs[slot];
        if (s.bytes < bytes) {
            if (s.p) TT_CUDA(cudaFree(s.p));
            s.p = nullptr;
            s.bytes = 0;
            size_t b = bytes < 256 ? 256 : bytes;
            b = (b + b / 8 + 255) & ~size_t(255);   // headroom against regrowth
            const bool inject = fail_in && --fail_in == 0;
            cudaError_t e = inject ? cudaErrorMemoryAllocation : cudaMalloc(&s.p, b);
            if (e != cudaSuccess) {
                cudaGetLastError();
                throw Error(TT_ERR_LENGTH, "device memory exhausted (" + std::to_string(b) + " bytes)");
            }
            s.bytes = b;
        }
        return s.p;
    }
    template <typename T>
    T* get(int slot, size_t count) { return static_cast<T*>(get(slot, count * sizeof(T))); }
    void release() {
        for (auto& s : slabs)
            if (s.p) cudaFree(s.p);
        slabs.clear();
    }
};

// Pinned host staging, grown on demand.
struct Pinned {
    void* p = nullptr;
    size_t bytes = 0;
    void* get(size_t b) {
        if (bytes < b) {
            if (p) cudaFreeHost(p);
            p = nullptr;
            b = (b + b / 8 + 4095) & ~size_t(4095);
            TT_CUDA(cudaMallocHost(&p, b));
            bytes = b;
        }
        return p;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
    }
};

// Arena slots. Each stage documents the slots it uses; a stage never holds a
// slot across a call into another stage that uses the same slot.
enum Slot : int {
    S_SORT_A = 0, S_SORT_B, S_SORT_HIST, S_SORT_VA, S_SORT_VB,   // radix sort
    S_SCAN, S_FLAGS, S_EDGE_KEYS, S_EDGE_TMP, S_COUNT,            // edges / compaction
    S_UF_PARENT, S_UF_BEST, S_UF_WORK, S_UF_WORK2,                // Borůvka
    S_MAT, S_PTS, S_OUT0, S_OUT1, S_OUT2, S_OUT3, S_OUT4, S_OUT5,         // host-buffer entry points
    S_KNN_D, S_KNN_I, S_GRAPH_KEYS, S_GRAPH_TMP, S_PIV,           // kNN / graph / pivots
    S_SCAN2, S_SCAN3, S_MISC0, S_MISC1, S_MISC2, S_MISC3, S_ROWMAX, S_GRAPH_RP, S_ASM0, S_ASM1, S_ASM2, S_ASM3, S_ASM4,
    S_TC_X, S_TC_PERM, S_TC_STATS, S_TC_KEYS, S_TC_VALS, S_TC_PIV,   // tensor-core kNN (tile order)
    S_TC_KEY2, S_TC_VAL2, S_TC_CELL, S_TC_LO, S_TC_ERR, S_TC_SPV,
    S_EDGE_CNT, S_EDGE_SORT, S_EDGE_IDX, S_EDGE_INV,               // ordered edge generation
    S_GRAPH_LONG, S_GRAPH_CI, S_GRAPH_W,                           // kNN graph: long rows; its columns and weights
    S_RZ_D, S_RZ_V,                                                // RedZeD edge lists sized to their count
    S_TXT, S_TXT_CNT, S_TXT_LINES, S_TXT_TOK, S_TXT_HOST,          // text ingestion
    S_DIM0_ERR,                                                    // dim0's announced-count check
    S_MST_KB, S_MST_Q,                                             // MST: interior bounds, scanned points
    S_NSLOTS
};

}  // namespace tt

// Opaque context behind the C-ABI.
struct tt_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    tt::Arena arena;
    tt::Pinned pinned;
    std::string last_error;
    int sms = tt::kSMs;
    double last_kernel_ms = 0.0;   // device time of the last stage (CUDA events)
    uint64_t launches = 0;          // kernels launched through this context
    int knn_mode = 0;               // 0 auto, 1 exhaustive scan, 2 tensor-core filter where applicable
    uint64_t memory_budget = 0;     // bytes a dense distance matrix may take (0: half the host's memory)
    uint64_t filter_evals = 0;      // exact evaluations the last tensor-core kNN let through
    uint64_t filter_tiles = 0;      // 128 x 128 Gram tiles the last tensor-core kNN computed
    cudaStream_t aux = nullptr;     // copies overlapped with compute (created on first use)
    cudaEvent_t aux_ev = nullptr;
    unsigned long long* tc_host = nullptr;   // page-locked: the tensor-core kNN's error word and counters
    bool tc_pending = false;                 // ... copied there, not yet read (deferred to a later sync)
    unsigned* fin_host = nullptr;   // mapped page-locked: the points' non-finite flag (check_finite_async)
    unsigned* fin_dev = nullptr;    // ... its device address
    cudaEvent_t fin_ev = nullptr;   // ... its copy recorded
    bool fin_pending = false;       // ... not yet read
    cudaStream_t side = nullptr;    // kernels overlapped with the main stream's (created on first use)
    cudaEvent_t side_ev[2] = {nullptr, nullptr};
};

namespace tt {
// The context's side stream (non-blocking, so it also runs beside a legacy
// default main stream; the device's highest priority, so its short kernels
// are scheduled ahead of the main stream's waiting blocks), ordered after
// everything issued so far on the main stream. Whoever forks work onto it
// joins it back (side_join) before the main stream reads the results.
inline cudaStream_t side_after_main(tt_ctx* c) {
    if (!c->side) {
        int least = 0, greatest = 0;
        TT_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        TT_CUDA(cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, greatest));
    }
    for (auto& e : c->side_ev)
        if (!e) TT_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    TT_CUDA(cudaEventRecord(c->side_ev[0], c->stream));
    TT_CUDA(cudaStreamWaitEvent(c->side, c->side_ev[0], 0));
    return c->side;
}
// The main stream waits for everything issued so far on the side stream.
inline void side_join(tt_ctx* c) {
    TT_CUDA(cudaEventRecord(c->side_ev[1], c->side));
    TT_CUDA(cudaStreamWaitEvent(c->stream, c->side_ev[1], 0));
}
// Joins on scope exit unless released; on an exception the side stream is
// drained instead, so no side kernel outlives the call that launched it.
struct SideScope {
    tt_ctx* c;
    bool open = false;
    explicit SideScope(tt_ctx* ctx) : c(ctx) {}
    cudaStream_t fork() {
        open = true;
        return side_after_main(c);
    }
    void join() {
        if (open) side_join(c);
        open = false;
    }
    ~SideScope() {
        if (open) cudaStreamSynchronize(c->side);
    }
};
}  // namespace tt
