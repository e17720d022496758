// ptx.cuh -- inline-PTX helpers for sm_103a: mbarriers, bulk (TMA) copies,
// proxy fences and bounded waits.
//
// Every wait here is bounded: after kWaitLimitNs of wall time (read from
// %globaltimer) it records DEV_ERR_TIMEOUT in the launch's status word and
// returns false (an mbarrier wait first gives its copies the same time again
// to land), so a kernel can never spin forever.
#pragma once

#include <cstdint>

#include "ginf_internal.h"

namespace ginf_gpu {

constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t global_timer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Makes the initialised barrier visible to the async proxy (bulk copies).
__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the barrier phase with the given parity.  After the time limit
// it records DEV_ERR_TIMEOUT and keeps waiting, for at most the same time
// again, so that copies still in flight land before the caller gives up and
// its shared memory is released; it then returns false, whether or not the
// phase completed in that second period.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, int *status) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_timer_ns();
    bool late = false;
    for (uint32_t n = 1;; ++n) {
        if (mbar_try_wait(bar, parity)) return !late;
        if ((n & 63u) == 0) {
            const uint64_t dt = global_timer_ns() - t0;
            if (!late && dt > kWaitLimitNs) {
                if (status) atomicOr(status, DEV_ERR_TIMEOUT);
                late = true;
            }
            if (dt > 2 * kWaitLimitNs) return false;
        }
    }
}

// Bulk copy global -> shared (this CTA), completion counted in bytes on bar.
// dst, src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_load(void *smem_dst, const void *gsrc, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(smem_dst)),
        "l"(gsrc), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// Bulk copy shared -> global, tracked by this thread's bulk async-groups.
__device__ __forceinline__ void bulk_store(void *gdst, const void *smem_src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst),
                 "r"(smem_addr(smem_src)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// This thread's bulk stores have finished reading shared memory.
__device__ __forceinline__ void bulk_wait_read_all() {
    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

// This thread's bulk stores are complete (globally performed).
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Orders this thread's generic-proxy shared-memory writes before later
// async-proxy (bulk copy) accesses.
__device__ __forceinline__ void fence_proxy_async_shared() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Orders this thread's async-proxy (bulk copy) and generic-proxy accesses to
// global memory.
__device__ __forceinline__ void fence_proxy_async_global() {
    asm volatile("fence.proxy.async.global;" ::: "memory");
}

// Programmatic dependent launch: the next kernel in the stream (launched
// with programmatic stream serialisation) may start now; it waits in
// grid_dependency_wait() until this grid has completed and its memory
// operations are visible.
__device__ __forceinline__ void launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Thread-block clusters: this CTA's coordinates inside its cluster, the
// cluster's shape, and the cluster's coordinates in the grid of clusters.
__device__ __forceinline__ uint32_t cluster_ctaid_x() {
    uint32_t v;
    asm("mov.u32 %0, %%cluster_ctaid.x;" : "=r"(v));
    return v;
}
__device__ __forceinline__ uint32_t cluster_ctaid_y() {
    uint32_t v;
    asm("mov.u32 %0, %%cluster_ctaid.y;" : "=r"(v));
    return v;
}
__device__ __forceinline__ uint32_t cluster_nctaid_x() {
    uint32_t v;
    asm("mov.u32 %0, %%cluster_nctaid.x;" : "=r"(v));
    return v;
}
__device__ __forceinline__ uint32_t cluster_nctaid_y() {
    uint32_t v;
    asm("mov.u32 %0, %%cluster_nctaid.y;" : "=r"(v));
    return v;
}
__device__ __forceinline__ uint32_t clusterid_x() {
    uint32_t v;
    asm("mov.u32 %0, %%clusterid.x;" : "=r"(v));
    return v;
}
__device__ __forceinline__ uint32_t clusterid_y() {
    uint32_t v;
    asm("mov.u32 %0, %%clusterid.y;" : "=r"(v));
    return v;
}

// The distributed-shared-memory address of the same offset in the shared
// memory of CTA `rank` of this cluster.
__device__ __forceinline__ uint32_t dsmem_addr(uint32_t local_smem_addr, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local_smem_addr), "r"(rank));
    return r;
}

// 16-byte store into (possibly another CTA's) shared memory of this cluster.
__device__ __forceinline__ void st_dsmem_v4(uint32_t addr, float a, float b, float c, float d) {
    asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "f"(a), "f"(b), "f"(c), "f"(d)
                 : "memory");
}

// Cluster-wide barrier: every thread of every CTA of the cluster arrives
// (release: its earlier shared-memory writes, local and remote, become
// visible) and waits (acquire).  Must be reached by all threads, convergently.
__device__ __forceinline__ void cluster_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Grid-wide barrier for a cooperative launch (all blocks co-resident).  bar
// holds {arrived, generation}, zeroed before the launch.  The last block to
// arrive resets the count and advances the generation; the others wait for
// the generation to change, each for at most kWaitLimitNs, then record
// DEV_ERR_TIMEOUT and report false (block-uniformly).
__device__ __forceinline__ bool grid_barrier(unsigned int *bar, unsigned int nblocks, int *status) {
    __syncthreads();
    int ok = 1;
    if (threadIdx.x == 0) {
        volatile unsigned int *vgen = bar + 1;
        const unsigned int gen = *vgen;
        __threadfence();
        const unsigned int arrived = atomicAdd(bar, 1u) + 1u;
        if (arrived == nblocks) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            const uint64_t t0 = global_timer_ns();
            while (*vgen == gen) {
                __nanosleep(64);
                if (global_timer_ns() - t0 > kWaitLimitNs) {
                    atomicOr(status, DEV_ERR_TIMEOUT);
                    ok = 0;
                    break;
                }
            }
        }
        __threadfence();
    }
    return __syncthreads_and(ok) != 0;
}

}  // namespace ginf_gpu
