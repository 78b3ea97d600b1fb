// Device-wide primitives: single-pass exclusive scan and a stable LSD radix
// sort, both with decoupled look-back across tiles (tiles take ids from an
// atomic counter in launch order, so every tile waits only on tiles that are
// already running).  Element counts may live in device memory so that the
// launches are fixed-size and graph-capturable; blocks past the live count
// exit at once.  Every spin-wait is bounded: on timeout the kernel records an
// error flag and returns without publishing or writing anything further (the
// host then fails the step).
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
// Iteration limit of every bounded wait (tile look-back, grid barrier, union
// retries, colouring passes).  Each translation unit holds its own
// __constant__ copy; setSpinLimit (prims.cu) writes all of them on the current
// device, and the waits read it at run time, so captured graphs see a change.
// A wait that runs out sets kErrTimeout, publishes nothing and its kernel
// returns at once; the step then fails with "a bounded wait timed out" and the
// world keeps its state from before the step.
constexpr uint32_t kSpinLimitDefault = 1u << 24;
namespace {
__constant__ uint32_t c_spinLimit = kSpinLimitDefault;
// Writes this translation unit's copy of the limit (host side).
inline void setSpinLimitOfUnit(uint32_t limit) {
    PE_CHECK(cudaMemcpyToSymbol(c_spinLimit, &limit, sizeof(limit)));
}
} // namespace
__device__ __forceinline__ uint32_t spinLimit() { return c_spinLimit; }


__device__ __forceinline__ uint32_t ldvol(const uint32_t *p) { return *(volatile const uint32_t *)p; }
__device__ __forceinline__ unsigned long long ldvol64(const unsigned long long *p) {
    return *(volatile const unsigned long long *)p;
}

// Look-back for one 32-bit counter per tile, done by one full warp.
// state[t] = (flag << 32) | value, flag 1 = tile aggregate, 2 = inclusive
// prefix.  Publishes the tile's aggregate, then each round reads the states of
// 32 predecessors at once (lane i: tile - 1 - base - i) and sums them up to the
// nearest inclusive prefix, so a walk over many finished tiles costs one
// memory round trip per 32 tiles.  Publishes the tile's inclusive prefix; every
// lane returns the exclusive prefix.  If the wait runs out, *timedOut is set
// on every lane, kErrTimeout is raised and no prefix is published (the tiles
// after this one run out as well); the caller's block then returns.
__device__ __forceinline__ uint32_t lookbackExclusiveWarp(unsigned long long *state, uint32_t tile,
                                                          uint32_t aggregate, uint32_t *err, bool *timedOut) {
    *timedOut = false;
    const uint32_t lane = threadIdx.x & 31;
    if (tile == 0) {
        if (lane == 0) atomicExch(&state[0], (2ull << 32) | aggregate);
        return 0;
    }
    if (lane == 0) atomicExch(&state[tile], (1ull << 32) | aggregate);
    uint32_t prefix = 0, spins = 0;
    int64_t base = (int64_t)tile - 1;
    while (base >= 0) {
        const int64_t t = base - (int64_t)lane;
        // Lanes before tile 0 read as an inclusive prefix of 0.
        const unsigned long long v = t >= 0 ? ldvol64(&state[t]) : (2ull << 32);
        const uint32_t flag = (uint32_t)(v >> 32);
        const uint32_t done = __ballot_sync(0xffffffffu, flag == 2);
        const uint32_t zero = __ballot_sync(0xffffffffu, flag == 0);
        const uint32_t first = done & (0u - done);           // nearest inclusive prefix
        const uint32_t upto = done ? (first << 1) - 1u : 0xffffffffu;
        if (zero & upto) {
            if (++spins > spinLimit()) {
                if (lane == 0) atomicOr(err, kErrTimeout);
                *timedOut = true;
                return 0;
            }
            continue;
        }
        uint32_t s = ((upto >> lane) & 1u) ? (uint32_t)v : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        prefix += s;
        if (done) break;
        base -= 32;
    }
    if (lane == 0) atomicExch(&state[tile], (2ull << 32) | (prefix + aggregate));
    return prefix;
}

// Block-wide exclusive scan of one value per thread (blockDim.x a multiple of
// 32, at most 256).
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
// only ever counts arrivals: the barrier a block arrives at ends when the
// count reaches the next multiple of the grid size, so the last block's
// arrival is the release (one atomic per block, no reset or generation word
// on the path).  Every kernel that shares the counter between two resets runs
// the same grid size and passes every barrier on every block.  Bounded spin:
// returns false on every thread of the block when its wait ran out
// (kErrTimeout raised), and the caller returns from the kernel at once.  The
// counter is reset before every solver pass that uses it.
__device__ __forceinline__ bool gridBarrier(uint32_t *bar, uint32_t *err) {
    __shared__ uint32_t s_barrierTimedOut;
    __syncthreads();
    if (threadIdx.x == 0) {
        s_barrierTimedOut = 0;
        __threadfence();
        const uint32_t arrived = atomicAdd(&bar[0], 1u);
        const uint32_t target = (arrived / gridDim.x + 1u) * gridDim.x;
        uint32_t spins = 0;
        while ((int32_t)(ldvol(&bar[0]) - target) < 0) {
            if (++spins > spinLimit()) {
                atomicOr(err, kErrTimeout);
                s_barrierTimedOut = 1;
                break;
            }
        }
        __threadfence();
    }
    __syncthreads();
    return s_barrierTimedOut == 0;
}

} // namespace pe
