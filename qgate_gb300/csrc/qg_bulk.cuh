// Shared-memory mbarriers and bulk async copies (cp.async.bulk) for sm_103a
// kernels.  Every mbarrier wait is bounded: it reports failure instead of
// spinning forever, and the caller records an error status.
#pragma once
#include <cstdint>

namespace qg {

__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}

// Makes barrier initialisation visible to the async proxy (bulk copies).
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(unsigned bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(bar) : "memory");
}

// Bounded wait for the completion of the phase with the given parity.  Each
// try suspends the thread until the phase completes or a 20 us hint runs
// out, so waiting threads do not spin on the issue slots; at most 2^16
// tries (about 1.3 s).
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
    for (int i = 0; i < (1 << 16); ++i) {
        unsigned ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity), "r"(20000u)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// Global -> shared copy of `bytes` (multiple of 16, both addresses 16-byte
// aligned) completing on `bar`, which this thread arms for the bytes.
__device__ __forceinline__ void bulk_load(unsigned dst, const void *src, unsigned bytes,
                                          unsigned bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
        "[%3];\n" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

// Shared -> global copy in the current bulk group.
__device__ __forceinline__ void bulk_store(void *dst, unsigned src, unsigned bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;\n" ::"l"(dst),
                 "r"(src), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_commit() {
    asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
}

// Until at most N committed groups still read their shared-memory source.
template <int N> __device__ __forceinline__ void bulk_wait_read() {
    asm volatile("cp.async.bulk.wait_group.read %0;\n" ::"n"(N) : "memory");
}

// Until at most N committed groups are incomplete.
template <int N> __device__ __forceinline__ void bulk_wait() {
    asm volatile("cp.async.bulk.wait_group %0;\n" ::"n"(N) : "memory");
}

// Orders this thread's shared-memory writes before later bulk copies.
__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

}  // namespace qg
