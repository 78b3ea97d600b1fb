// Island-parallel sweeps of the multi-kernel solver (more manifolds than the
// cluster solver holds).  The colouring is the global one (k_color); the
// sweeps then run island by island instead of colour by colour across the
// whole grid: manifolds joined by a dynamic body form an island (static bodies
// join nothing, sequential_impulse_solver.cpp:366-442), no two islands share a
// body, so each island can be solved on its own in the global (colour, index)
// order restricted to it — bit for bit the grid-wide sweeps, without a grid
// barrier per colour.
//
//   k_isl_init  : every dynamic endpoint its own island
//   k_isl_unite : union of the bodies of every solved manifold with two dynamic
//                 bodies (lock-free; roots are the smallest body index)
//   k_isl_count : each solved manifold's island and slot in it; islands listed
//   k_isl_fill  : manifolds into their islands' lists (offsets from a scan);
//                 islands of 32 manifolds or more queued before the others
//   k_isl_solve : one warp per island (large ones first, from a queue): the
//                 island's manifolds sorted by (colour, index), then warm start
//                 and iterations colour by colour with __syncwarp; manifolds
//                 without a dynamic body (nothing to share) are solved alone
#include "pe_kernels.cuh"
#include "pe_prims.cuh"
#include "pe_solve.cuh"
#include "pe_stages.h"

namespace pe {

namespace {

constexpr int kIslThreads = 128;           // four warps per block
constexpr uint32_t kIslWarpSort = 1024;    // island keys sorted in shared memory up to this size
constexpr uint32_t kIslNone = 0xFFFFFFFFu;

inline uint32_t islGrid(uint32_t n) {
    const uint32_t b = (n + kIslThreads - 1) / kIslThreads;
    return b ? (b < 152u * 16u ? b : 152u * 16u) : 1u;
}

__device__ __forceinline__ uint32_t islFind(const uint32_t *par, uint32_t i, uint32_t nb) {
    for (uint32_t n = 0; n <= nb; ++n) {
        const uint32_t p = ldvol(&par[i]);
        if (p == i) return i;
        i = p;
    }
    return i;
}

__device__ __forceinline__ void islUnite(uint32_t *par, uint32_t a, uint32_t b, uint32_t nb, uint32_t *err) {
    for (uint32_t spins = 0; spins < kSpinLimit; ++spins) {
        a = islFind(par, a, nb);
        b = islFind(par, b, nb);
        if (a == b) return;
        const uint32_t hi = a > b ? a : b, lo = a > b ? b : a;
        const uint32_t old = atomicCAS(&par[hi], hi, lo);
        if (old == hi) return;
        a = old;
        b = lo;
    }
    atomicOr(err, kErrTimeout);
}

__device__ __forceinline__ uint32_t *islPar(const SolveArgs &a) { return a.sb.islPar; }
__device__ __forceinline__ uint32_t *islCnt(const SolveArgs &a) { return a.sb.islPar + a.w.nb; }

} // namespace

// Per-body counts all zero (they are scanned into list offsets), every dynamic
// endpoint its own island.
__global__ void k_isl_init(SolveArgs a) {
    const uint32_t M = min(*a.count, a.mcap);
    uint32_t *par = islPar(a), *cnt = islCnt(a);
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    if (t < 8) a.sb.islCounters[t] = 0u;
    for (uint32_t i = t; i < a.w.nb; i += stride) cnt[i] = 0u;
    for (uint32_t m = t; m < M; m += stride) {
        const uint32_t fl = a.sb.dyn[m];
        if (fl & kFlagDynA) par[a.mv.bodyA[m]] = a.mv.bodyA[m];
        if (fl & kFlagDynB) par[a.mv.bodyB[m]] = a.mv.bodyB[m];
    }
}

__global__ void k_isl_unite(SolveArgs a) {
    const uint32_t M = min(*a.count, a.mcap);
    uint32_t *par = islPar(a);
    for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
        const uint32_t fl = a.sb.dyn[m];
        if ((fl & (kFlagValid | kFlagDynA | kFlagDynB)) == (kFlagValid | kFlagDynA | kFlagDynB))
            islUnite(par, a.mv.bodyA[m], a.mv.bodyB[m], a.w.nb, &a.st->err);
    }
}

// islCounters: [0] islands, [1] lone manifolds (solved, no dynamic body),
// [2] work queue of k_isl_solve, [3] listed manifolds, [4] / [5] large / small
// islands queued.
__global__ void k_isl_count(SolveArgs a) {
    const uint32_t M = min(*a.count, a.mcap);
    uint32_t *par = islPar(a), *cnt = islCnt(a);
    for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
        const uint32_t fl = a.sb.dyn[m];
        uint32_t root = kIslNone;
        if ((fl & kFlagValid) && (fl & (kFlagDynA | kFlagDynB))) {
            root = islFind(par, (fl & kFlagDynA) ? a.mv.bodyA[m] : a.mv.bodyB[m], a.w.nb);
            const uint32_t pos = atomicAdd(&cnt[root], 1u);
            a.sb.islSlot[m] = pos;
            if (pos == 0) a.sb.islRoots[atomicAdd(&a.sb.islCounters[0], 1u)] = root;
        } else if (fl & kFlagValid) {
            a.sb.islLone[atomicAdd(&a.sb.islCounters[1], 1u)] = m;
        }
        a.sb.islRoot[m] = root;
    }
}

__global__ void k_isl_fill(SolveArgs a) {
    const uint32_t M = min(*a.count, a.mcap);
    const uint32_t *cnt = islCnt(a);
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    for (uint32_t m = t; m < M; m += stride) {
        const uint32_t r = a.sb.islRoot[m];
        if (r != kIslNone) a.sb.islList[a.sb.islOff[r] + a.sb.islSlot[m]] = m;
    }
    // the queue: islands of 32 manifolds or more at the front (a warp's
    // lanes all busy; they bound the sweep), the others behind them
    uint32_t *queue = reinterpret_cast<uint32_t *>(a.sb.islKeys);
    const uint32_t nIsl = a.sb.islCounters[0];
    for (uint32_t i = t; i < nIsl; i += stride) {
        const uint32_t r = a.sb.islRoots[i];
        if (cnt[r] >= 32) queue[atomicAdd(&a.sb.islCounters[4], 1u)] = r;
        else queue[nIsl - 1 - atomicAdd(&a.sb.islCounters[5], 1u)] = r;
    }
}

namespace {
// Sorts keys[0, n) (n a power of two) ascending with one warp.
__device__ __forceinline__ void warpBitonicSort(unsigned long long *keys, uint32_t n, uint32_t lane) {
    for (uint32_t k = 2; k <= n; k <<= 1)
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = lane; i < n; i += 32) {
                const uint32_t ixj = i ^ j;
                if (ixj > i) {
                    const unsigned long long x = keys[i], y = keys[ixj];
                    if ((x > y) == ((i & k) == 0)) {
                        keys[i] = y;
                        keys[ixj] = x;
                    }
                }
            }
            __syncwarp();
        }
}
} // namespace

__global__ void __launch_bounds__(kIslThreads) k_isl_solve(SolveArgs a) {
    __shared__ unsigned long long s_keys[kIslThreads / 32][kIslWarpSort];
    __shared__ uint32_t s_start[kIslThreads / 32][kMaxColors + 1];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t nIsl = a.sb.islCounters[0];
    for (;;) {
        uint32_t i = 0;
        if (lane == 0) i = atomicAdd(&a.sb.islCounters[2], 1u);
        i = __shfl_sync(0xffffffffu, i, 0);
        if (i >= nIsl) break;
        const uint32_t r = reinterpret_cast<const uint32_t *>(a.sb.islKeys)[i];
        const uint32_t n = islCnt(a)[r], base = a.sb.islOff[r];
        // the island's manifolds in (colour, index) order
        const uint32_t n2 = nextPow2(n);
        // large islands sort in global scratch: [2 base, 2 base + n2) lies
        // inside the island's own range [2 base, 2 (base + n)) of 2 mcap keys
        unsigned long long *keys = n2 <= kIslWarpSort ? s_keys[warp] : a.sb.islSort + (size_t)2 * base;
        for (uint32_t j = lane; j < n2; j += 32) {
            unsigned long long key = ~0ull;
            if (j < n) {
                const uint32_t m = a.sb.islList[base + j];
                key = ((unsigned long long)a.sb.color[m] << 32) | m;
            }
            keys[j] = key;
        }
        __syncwarp();
        warpBitonicSort(keys, n2, lane);
        // colour ranges [s_start[c], s_start[c + 1])
        const uint32_t lastColor = (uint32_t)(keys[n - 1] >> 32);
        const uint32_t C = lastColor < (uint32_t)kMaxColors ? lastColor + 1 : (uint32_t)kMaxColors;
        for (uint32_t c = lane; c <= C; c += 32) {
            uint32_t lo = 0, hi = n;
            while (lo < hi) {
                const uint32_t mid = (lo + hi) >> 1;
                if ((uint32_t)(keys[mid] >> 32) < c) lo = mid + 1;
                else hi = mid;
            }
            s_start[warp][c] = lo;
        }
        __syncwarp();
        for (int pass = 0; pass <= a.iterations; ++pass)
            for (uint32_t c = 0; c < C; ++c) {
                for (uint32_t j = s_start[warp][c] + lane; j < s_start[warp][c + 1]; j += 32) {
                    const uint32_t m = (uint32_t)(keys[j] & 0xFFFFFFFFull);
                    if (pass == 0) warmStartOne(a, j, m);
                    else solveOneChained(a, j, m);
                }
                __syncwarp();
            }
        __syncwarp();
    }
    // manifolds with no dynamic body: nothing is shared, each alone
    const uint32_t nLone = a.sb.islCounters[1];
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < nLone; j += gridDim.x * blockDim.x) {
        const uint32_t m = a.sb.islLone[j];
        warmStartOne(a, j, m);
        for (int it = 0; it < a.iterations; ++it) solveOne(a, j, m);
    }
}

void launchSolveIslands(const SolveArgs &a, Scratch &ws, cudaStream_t s) {
    const uint32_t mcap = a.mcap;
    k_isl_init<<<islGrid(mcap), kIslThreads, 0, s>>>(a);
    PE_LAUNCHED();
    k_isl_unite<<<islGrid(mcap), kIslThreads, 0, s>>>(a);
    PE_LAUNCHED();
    k_isl_count<<<islGrid(mcap), kIslThreads, 0, s>>>(a);
    PE_LAUNCHED();
    // offsets of the islands' lists: exclusive scan of the per-body counts
    // (zero for bodies that are not an island root)
    launchScanExclusive(a.sb.islPar + a.w.nb, a.sb.islOff, nullptr, a.w.nb, &a.sb.islCounters[3], ws, &a.st->err, s);
    k_isl_fill<<<islGrid(mcap), kIslThreads, 0, s>>>(a);
    PE_LAUNCHED();
    k_isl_solve<<<152 * 4, kIslThreads, 0, s>>>(a);
    PE_LAUNCHED();
}

} // namespace pe
