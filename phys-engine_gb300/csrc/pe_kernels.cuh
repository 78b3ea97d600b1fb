// Common includes for the step kernels.
#pragma once
#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>

#include "pe_engine.h"
#include "pe_math.cuh"
#include "pe_prims.cuh"

namespace pe {

// Warp-aggregated append: one atomic per converged group of lanes.
__device__ __forceinline__ uint32_t aggregatedAppend(uint32_t *counter) {
    namespace cg = cooperative_groups;
    cg::coalesced_group g = cg::coalesced_threads();
    uint32_t base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(counter, g.size());
    return g.shfl(base, 0) + g.thread_rank();
}

__device__ __forceinline__ void aggregatedAdd64(unsigned long long *counter, unsigned long long v) {
    namespace cg = cooperative_groups;
    cg::coalesced_group g = cg::coalesced_threads();
    unsigned long long s = cg::reduce(g, v, cg::plus<unsigned long long>());
    if (g.thread_rank() == 0 && s) atomicAdd(counter, s);
}

__device__ __forceinline__ void aggregatedAdd32(uint32_t *counter, uint32_t v) {
    namespace cg = cooperative_groups;
    cg::coalesced_group g = cg::coalesced_threads();
    const uint32_t s = cg::reduce(g, v, cg::plus<uint32_t>());
    if (g.thread_rank() == 0 && s) atomicAdd(counter, s);
}

// Maximum into *counter: one atomic per converged group of lanes.
__device__ __forceinline__ void aggregatedMax32(uint32_t *counter, uint32_t v) {
    namespace cg = cooperative_groups;
    cg::coalesced_group g = cg::coalesced_threads();
    const uint32_t mx = cg::reduce(g, v, cg::greater<uint32_t>());
    if (g.thread_rank() == 0) atomicMax(counter, mx);
}

// Adds 1 to counters[key] once per group of converged lanes sharing the key.
__device__ __forceinline__ void aggregatedCount(unsigned long long *counters, uint32_t key) {
    const uint32_t active = __activemask();
    const uint32_t peers = __match_any_sync(active, key);
    const int leader = __ffs(peers) - 1;
    if ((int)(threadIdx.x & 31) == leader) atomicAdd(&counters[key], (unsigned long long)__popc(peers));
}

// Appends to counters[key]: one atomic per group of converged lanes sharing
// the key; returns the lane's slot.
__device__ __forceinline__ uint32_t aggregatedAppendKeyed(uint32_t *counters, uint32_t key) {
    const uint32_t active = __activemask();
    const uint32_t peers = __match_any_sync(active, key);
    const uint32_t lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if ((int)lane == leader) base = atomicAdd(&counters[key], (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + __popc(peers & ((1u << lane) - 1u));
}

// Counters of a new step: all zero, the bound count, empty grid bounds.
__device__ __forceinline__ unsigned long long globalNs() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void initStepStats(DevStats *st, uint32_t inputCount) {
    memset(st, 0, offsetof(DevStats, stamp));  // the stage stamps are kept
    st->inputCount = inputCount;
    for (int a = 0; a < 3; ++a) {
        st->cellLo[a] = 0x7FFFFFFF;
        st->cellHi[a] = (int32_t)0x80000000;
    }
}

} // namespace pe
