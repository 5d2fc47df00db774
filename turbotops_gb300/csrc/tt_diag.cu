// tt_diag.cu — failure-detection self-test (no reference counterpart).
//
// Every device wait in this library is bounded: a wait that runs out records
// TT_DEV_ERR_TIMEOUT in the launch's error word and the kernel returns, so
// the host gets TT_ERR_TIMEOUT and the context stays usable. This kernel
// exercises exactly that path on purpose, without any fault: one thread
// initialises an mbarrier that expects one arrival nobody makes and waits on
// it with a short poll limit; the wait runs out, the error word is set, the
// kernel ends normally.
#include "tt_internal.cuh"
#include "tt_tma.cuh"

using namespace tt;

namespace {

__global__ void k_wait_nobody(u32 polls, u32* __restrict__ err) {
    __shared__ __align__(8) u64 bar;
    if (threadIdx.x != 0) return;
    mbar_init(&bar, 1);
    fence_mbar_init();
    const u32 a = smem_addr(&bar);
    for (u32 i = 0; i < polls; ++i) {
        u32 done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(0u)
            : "memory");
        if (done) return;
    }
    atomicOr(err, TT_DEV_ERR_TIMEOUT);
}

}  // namespace

namespace tt {
void selftest_wait_timeout(tt_ctx* c, u32 polls) {
    if (polls == 0 || polls > (1u << 20)) invalid("gb300: self-test poll limit must be in [1, 2^20]");
    u32* e = c->arena.get<u32>(S_MISC2, 4);
    TT_CUDA(cudaMemsetAsync(e, 0, sizeof(u32), c->stream));
    k_wait_nobody<<<1, 32, 0, c->stream>>>(polls, e);
    TT_LAUNCH("k_wait_nobody");
    ++c->launches;
    u32 h = 0;
    TT_CUDA(cudaMemcpyAsync(&h, e, 4, cudaMemcpyDeviceToHost, c->stream));
    TT_CUDA(cudaStreamSynchronize(c->stream));
    if (h & TT_DEV_ERR_TIMEOUT) throw Error(TT_ERR_TIMEOUT, "gb300: a bounded device wait timed out (self-test)");
}
}  // namespace tt
