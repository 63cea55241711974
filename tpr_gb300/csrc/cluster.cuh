// Thread-block cluster primitives (inline PTX, sm_90+; used on sm_103a):
// rank queries, the cluster-wide barrier, and asynchronous stores into
// another CTA's shared memory (distributed shared memory) that complete on
// an mbarrier there.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace tprgb {
namespace cl {

__device__ __forceinline__ unsigned rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

__device__ __forceinline__ unsigned size() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}

// Every thread of every CTA of the cluster arrives (release) and waits
// (acquire): shared-memory writes before it, to this CTA's or another
// CTA's shared memory, are visible to every CTA of the cluster after it.  All threads of the cluster must execute
// the same sequence of these barriers.
__device__ __forceinline__ void sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
                 "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Address of `p` (this CTA's shared memory) in CTA `r` of the cluster.
__device__ __forceinline__ uint32_t map(const void *p, unsigned r) {
    uint32_t a = (uint32_t)__cvta_generic_to_shared(p), out;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(out) : "r"(a), "r"(r));
    return out;
}

// Asynchronous 16-byte store into a CTA's shared memory (addr from map())
// that completes 16 bytes of transaction count on the mbarrier at `mbar`
// (map()ped into the same CTA).
__device__ __forceinline__ void st_async4(uint32_t addr, float4 v, uint32_t mbar) {
    asm volatile(
        "st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.f32 [%0], "
        "{%1, %2, %3, %4}, [%5];"
        :
        : "r"(addr), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w), "r"(mbar)
        : "memory");
}

// Wait, with cluster-scope acquire, for phase parity `phase` of an mbarrier
// in this CTA's shared memory that other CTAs' st_async4 complete; false
// after `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned phase, unsigned limit) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(bar);
    for (unsigned i = 0; i < limit; i++) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(a), "r"(phase)
            : "memory");
        if (ok) return true;
        if (i > 64) __nanosleep(64);
    }
    return false;
}

}  // namespace cl
}  // namespace tprgb
