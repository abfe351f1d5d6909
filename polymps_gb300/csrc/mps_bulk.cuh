// mps_bulk.cuh — shared-memory staging by the bulk-copy engine on sm_103a: mbarrier
// initialisation, transaction-count arrival, bounded parity waits, and the 1D global-to-
// shared bulk copy (cp.async.bulk; both addresses 16-byte aligned, the size a multiple of
// 16 bytes).
#pragma once

__device__ __forceinline__ unsigned smemAddr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbarInit(unsigned long long* b, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbarExpectTx(unsigned long long* b, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbarArrive(unsigned long long* b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smemAddr(b)) : "memory");
}
__device__ __forceinline__ bool mbarTry(unsigned long long* b, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smemAddr(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait (at most spins polls); false when it ran out
__device__ __forceinline__ bool mbarWaitN(unsigned long long* b, unsigned parity, int spins) {
    for (int k = 0; k < spins; k++)
        if (mbarTry(b, parity)) return true;
    return false;
}
__device__ __forceinline__ void bulkG2S(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smemAddr(dst)),
                 "l"(src), "r"(bytes), "r"(smemAddr(bar))
                 : "memory");
}
