// Thread-block cluster primitives (inline PTX, sm_90+; used on sm_103a):
// rank queries, the cluster-wide barrier, and stores to another CTA's
// shared memory (distributed shared memory).
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

__device__ __forceinline__ void st4(uint32_t addr, float4 v) {
    asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};"
                 :
                 : "r"(addr), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
                 : "memory");
}

}  // namespace cl
}  // namespace tprgb
