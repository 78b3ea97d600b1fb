// Device-wide primitives: single-pass exclusive scan and a stable LSD radix
// sort, both with decoupled look-back across tiles (tiles take ids from an
// atomic counter in launch order, so every tile waits only on tiles that are
// already running).  Element counts may live in device memory so that the
// launches are fixed-size and graph-capturable; blocks past the live count
// exit at once.  Every spin-wait is bounded: on timeout the kernel records an
// error flag and finishes without waiting (results are then invalid and the
// host reports PE_ERR_TIMEOUT).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "pe_engine.h"

namespace pe {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;       // 2048
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortRounds = 8;
constexpr int kSortTile = kSortThreads * kSortRounds;      // 2048
constexpr uint32_t kSpinLimit = 1u << 24;


__device__ __forceinline__ uint32_t ldvol(const uint32_t *p) { return *(volatile const uint32_t *)p; }
__device__ __forceinline__ unsigned long long ldvol64(const unsigned long long *p) {
    return *(volatile const unsigned long long *)p;
}

// Look-back for one 32-bit counter per tile.  state[t] = (flag << 32) | value,
// flag 1 = tile aggregate, 2 = inclusive prefix.  Returns the exclusive prefix
// of `tile` and publishes its inclusive prefix.  Called by one thread.
__device__ __forceinline__ uint32_t lookbackExclusive(unsigned long long *state, uint32_t tile, uint32_t aggregate,
                                                      uint32_t *err) {
    if (tile == 0) {
        atomicExch(&state[0], (2ull << 32) | aggregate);
        return 0;
    }
    atomicExch(&state[tile], (1ull << 32) | aggregate);
    uint32_t prefix = 0;
    int64_t t = (int64_t)tile - 1;
    uint32_t spins = 0;
    while (t >= 0) {
        unsigned long long v = ldvol64(&state[t]);
        uint32_t flag = (uint32_t)(v >> 32);
        if (flag == 0) {
            if (++spins > kSpinLimit) {
                atomicOr(err, kErrTimeout);
                break;
            }
            continue;
        }
        prefix += (uint32_t)v;
        if (flag == 2) break;
        --t;
    }
    atomicExch(&state[tile], (2ull << 32) | (prefix + aggregate));
    return prefix;
}

// Block-wide exclusive scan of one value per thread (blockDim.x == 256).
__device__ __forceinline__ uint32_t blockExclusiveScan(uint32_t v, uint32_t &total, uint32_t *smem /*[9]*/) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t n = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += n;
    }
    if (lane == 31) smem[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (int)(blockDim.x >> 5) ? smem[lane] : 0;
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t n = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += n;
        }
        if (lane < (int)(blockDim.x >> 5)) smem[lane] = wi - w;
        if (lane == (int)(blockDim.x >> 5) - 1) smem[8] = wi;
    }
    __syncthreads();
    uint32_t r = smem[warp] + incl - v;
    total = smem[8];
    __syncthreads();
    return r;
}

// Dynamic tile id, broadcast through shared memory.
__device__ __forceinline__ uint32_t takeTile(uint32_t *counter, uint32_t *slot) {
    if (threadIdx.x == 0) *slot = atomicAdd(counter, 1u);
    __syncthreads();
    uint32_t t = *slot;
    __syncthreads();
    return t;
}

// Grid-wide barrier for cooperative launches (all blocks co-resident).  bar[0]
// counts arrivals, bar[1] is the generation.  Bounded spin; on timeout the
// error flag is set and the block continues.
__device__ __forceinline__ void gridBarrier(uint32_t *bar, uint32_t *err) {
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t gen = ldvol(&bar[1]);
        __threadfence();
        uint32_t arrived = atomicAdd(&bar[0], 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(&bar[0], 0u);
            __threadfence();
            atomicAdd(&bar[1], 1u);
        } else {
            uint32_t spins = 0;
            while (ldvol(&bar[1]) == gen) {
                if (++spins > kSpinLimit) {
                    atomicOr(err, kErrTimeout);
                    break;
                }
            }
        }
        __threadfence();
    }
    __syncthreads();
}

} // namespace pe
