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
//   k_isl_solve : islands of kIslBlock to kIslBlockMax manifolds one thread
//                 block each (a pyramid of boxes), sorted by (colour, index) in
//                 shared memory and swept colour by colour with __syncthreads;
//                 then one warp per smaller island (those of 32 manifolds or
//                 more first, from a queue), swept with __syncwarp; islands of
//                 fewer than kIslThread manifolds one per thread, manifold
//                 after manifold in that order (a stack of two boxes would
//                 leave 30 lanes idle); manifolds without a dynamic body
//                 (nothing to share) are solved alone
//   k_isl_solve_large : when some island has more than kIslBlockMax
//                 manifolds (a settled pile), all islands together in
//                 grid-wide colour sweeps instead: the manifolds bucketed by
//                 colour, a grid barrier per colour.  Manifolds of one colour
//                 share no dynamic body, so their order inside a colour does
//                 not change the result.
#include <stdexcept>

#include "pe_block.cuh"
#include "pe_kernels.cuh"
#include "pe_prims.cuh"
#include "pe_solve.cuh"
#include "pe_stages.h"

namespace pe {

namespace {

constexpr int kIslThreads = 128;           // four warps per block
constexpr uint32_t kIslWarpSort = 1024;    // island keys sorted in shared memory up to this size
constexpr uint32_t kIslNone = 0xFFFFFFFFu;
// Islands of kIslBlock manifolds or more are swept by a whole thread block
// (one warp would take them colour by colour 32 manifolds at a time), up to
// kIslBlockMax manifolds (the block's shared key buffer).  An island above
// that (a settled pile of thousands of bodies) sends every island of the step
// to the grid-wide sweeps: measured on piles of 5,000 and 10,000 bodies,
// keeping the smaller islands apart only adds their sweep time to the grid's.
constexpr uint32_t kIslBlock = 512;
constexpr uint32_t kIslBlockMax = 4 * kIslWarpSort;
constexpr uint32_t kIslThread = 8;         // islands of fewer manifolds: one thread each
// islCounters: [0] islands, [1] lone manifolds (solved, no dynamic body), [2]
// work queue of the warp items, [3] listed manifolds, [4] / [5] islands of 32
// manifolds or more / kIslThread to 31 queued, [6] smaller islands, [7] set
// when an island exceeds kIslBlockMax manifolds, [8] block islands queued,
// [9] work queue of the block islands; [kIslColorCount + c] manifolds of
// colour c in the grid-wide sweeps, [kIslColorFill + c] their fill cursors
constexpr uint32_t kIslColorCount = 10;
constexpr uint32_t kIslColorFill = 10 + kMaxColors;
static_assert(kIslColorFill + kMaxColors == kIslCounterWords, "island counter layout");

inline uint32_t islGrid(uint32_t n) {
    const uint32_t b = (n + kIslThreads - 1) / kIslThreads;
    const uint32_t maxGrid = 16u * (uint32_t)smCount();
    return b ? (b < maxGrid ? b : maxGrid) : 1u;
}

// Root of i's island, halving the path on the way (par[i] = grandparent).
// Safe beside concurrent unions: only non-roots are written, a non-root
// never becomes a root again, and a grandparent stays an ancestor.
__device__ __forceinline__ uint32_t islFind(uint32_t *par, uint32_t i, uint32_t nb) {
    for (uint32_t n = 0; n <= nb; ++n) {
        const uint32_t p = ldvol(&par[i]);
        if (p == i) return i;
        const uint32_t gp = ldvol(&par[p]);
        if (gp == p) return p;
        par[i] = gp;
        i = gp;
    }
    return i;
}

__device__ __forceinline__ void islUnite(uint32_t *par, uint32_t a, uint32_t b, uint32_t nb, uint32_t *err) {
    for (uint32_t spins = 0; spins < spinLimit(); ++spins) {
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

// More colours than the per-colour counters hold (colour windows): every
// island goes to the grid-wide sweeps, with its per-colour counts and fill
// cursors in sb.colorStart.
__device__ __forceinline__ uint32_t islWideColors(const SolveArgs &a, uint32_t M) {
    const uint32_t C = __ldcg(&a.st->colors);
    return C > (uint32_t)kMaxColors ? (C < M ? C : M) : 0u;
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
    for (uint32_t i = t; i < kIslCounterWords; i += stride) a.sb.islCounters[i] = 0u;
    for (uint32_t i = t; i < a.w.nb; i += stride) cnt[i] = 0u;
    const uint32_t wideC = islWideColors(a, M);
    for (uint32_t i = t; i < wideC; i += stride) a.sb.colorStart[i] = 0u;
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

__global__ void k_isl_count(SolveArgs a) {
    const uint32_t M = min(*a.count, a.mcap);
    uint32_t *par = islPar(a), *cnt = islCnt(a);
    for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
        const uint32_t fl = a.sb.dyn[m];
        uint32_t root = kIslNone;
        if ((fl & kFlagValid) && (fl & (kFlagDynA | kFlagDynB))) {
            root = islFind(par, (fl & kFlagDynA) ? a.mv.bodyA[m] : a.mv.bodyB[m], a.w.nb);
            const uint32_t pos = aggregatedAppendKeyed(cnt, root);
            a.sb.islSlot[m] = pos;
            if (pos == kIslBlockMax) a.sb.islCounters[7] = 1u;
            if (pos == 0) a.sb.islRoots[aggregatedAppend(&a.sb.islCounters[0])] = root;
        } else if (fl & kFlagValid) {
            a.sb.islLone[aggregatedAppend(&a.sb.islCounters[1])] = m;
        }
        a.sb.islRoot[m] = root;
    }
}

// Islands of at least this many manifolds go to the grid-wide sweeps: all
// once some island is large or the colours exceed kMaxColors, none otherwise.
__device__ __forceinline__ uint32_t islSweepFrom(const SolveArgs &a, uint32_t M) {
    return (a.sb.islCounters[7] || islWideColors(a, M)) ? 1u : kIslNone;
}

__global__ void k_isl_fill(SolveArgs a) {
    const uint32_t M = min(*a.count, a.mcap);
    const uint32_t *cnt = islCnt(a);
    const uint32_t sweepFrom = islSweepFrom(a, M), wideC = islWideColors(a, M);
    uint32_t *colorCounts = wideC ? a.sb.colorStart : a.sb.islCounters + kIslColorCount;
    const uint32_t colorLimit = wideC ? wideC : (uint32_t)kMaxColors;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    for (uint32_t m = t; m < M; m += stride) {
        const uint32_t r = a.sb.islRoot[m];
        if (r == kIslNone) continue;
        a.sb.islList[a.sb.islOff[r] + a.sb.islSlot[m]] = m;
        const uint32_t c = a.sb.color[m];
        if (cnt[r] >= sweepFrom && c < colorLimit) aggregatedAppendKeyed(colorCounts, c);
    }
    // the warp queue: islands of 32 manifolds or more at the front (a warp's
    // lanes all busy; they bound the sweep), those of kIslThread to 31 from
    // the back; smaller ones to the per-thread list, islands of kIslBlock or
    // more to the block list (the per-thread list's area, from its end)
    uint32_t *queue = reinterpret_cast<uint32_t *>(a.sb.islKeys), *tiny = queue + a.mcap;
    const uint32_t nIsl = a.sb.islCounters[0];
    for (uint32_t i = t; i < nIsl; i += stride) {
        const uint32_t r = a.sb.islRoots[i];
        if (cnt[r] >= sweepFrom) continue;
        if (cnt[r] >= kIslBlock) tiny[a.mcap - 1 - aggregatedAppend(&a.sb.islCounters[8])] = r;
        else if (cnt[r] >= 32) queue[aggregatedAppend(&a.sb.islCounters[4])] = r;
        else if (cnt[r] >= kIslThread) queue[nIsl - 1 - aggregatedAppend(&a.sb.islCounters[5])] = r;
        else tiny[aggregatedAppend(&a.sb.islCounters[6])] = r;
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
    __shared__ uint32_t s_item;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // islands of kIslBlock manifolds or more: one block each
    {
        const uint32_t nBlock = a.sb.islCounters[8];
        const uint32_t *blockList = reinterpret_cast<const uint32_t *>(a.sb.islKeys) + a.mcap;
        unsigned long long *keys = &s_keys[0][0];  // kIslBlockMax keys
        uint32_t *start = s_start[0];
        for (;;) {
            if (threadIdx.x == 0) s_item = atomicAdd(&a.sb.islCounters[9], 1u);
            __syncthreads();
            const uint32_t item = s_item;
            if (item >= nBlock) break;
            const uint32_t r = blockList[a.mcap - 1 - item];
            const uint32_t n = islCnt(a)[r], base = a.sb.islOff[r];
            const uint32_t n2 = nextPow2(n);
            for (uint32_t j = threadIdx.x; j < n2; j += blockDim.x) {
                unsigned long long key = ~0ull;
                if (j < n) {
                    const uint32_t m = a.sb.islList[base + j];
                    key = ((unsigned long long)a.sb.color[m] << 32) | m;
                }
                keys[j] = key;
            }
            __syncthreads();
            blockBitonicSort(keys, n2);
            // colour ranges [start[c], start[c + 1])
            const uint32_t lastColor = (uint32_t)(keys[n - 1] >> 32);
            const uint32_t C = lastColor < (uint32_t)kMaxColors ? lastColor + 1 : (uint32_t)kMaxColors;
            for (uint32_t c = threadIdx.x; c <= C; c += blockDim.x) {
                uint32_t lo = 0, hi = n;
                while (lo < hi) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if ((uint32_t)(keys[mid] >> 32) < c) lo = mid + 1;
                    else hi = mid;
                }
                start[c] = lo;
            }
            __syncthreads();
            for (int pass = 0; pass <= a.iterations; ++pass)
                for (uint32_t c = 0; c < C; ++c) {
                    for (uint32_t j = start[c] + threadIdx.x; j < start[c + 1]; j += blockDim.x) {
                        const uint32_t m = (uint32_t)(keys[j] & 0xFFFFFFFFull);
                        if (pass == 0) warmStartOne(a, j, m);
                        else solveOneChained(a, j, m);
                    }
                    __syncthreads();
                }
        }
    }
    const uint32_t nIsl = a.sb.islCounters[0];
    const uint32_t nFront = a.sb.islCounters[4], nWarp = nFront + a.sb.islCounters[5], nTiny = a.sb.islCounters[6];
    const uint32_t nItems = nWarp + (nTiny + 31) / 32;
    const uint32_t *queue = reinterpret_cast<const uint32_t *>(a.sb.islKeys), *tiny = queue + a.mcap;
    for (;;) {
        uint32_t i = 0;
        if (lane == 0) i = atomicAdd(&a.sb.islCounters[2], 1u);
        i = __shfl_sync(0xffffffffu, i, 0);
        if (i >= nItems) break;
        if (i >= nWarp) {
            // 32 small islands, one per lane, each swept manifold after
            // manifold in (colour, index) order
            const uint32_t t = (i - nWarp) * 32 + lane;
            if (t < nTiny) {
                const uint32_t r = tiny[t];
                const uint32_t n = islCnt(a)[r], base = a.sb.islOff[r];
                unsigned long long *keys = &s_keys[warp][lane * kIslThread];
                for (uint32_t j = 0; j < n; ++j) {
                    const uint32_t m = a.sb.islList[base + j];
                    const unsigned long long key = ((unsigned long long)a.sb.color[m] << 32) | m;
                    uint32_t p = j;
                    for (; p > 0 && keys[p - 1] > key; --p) keys[p] = keys[p - 1];
                    keys[p] = key;
                }
                for (int pass = 0; pass <= a.iterations; ++pass)
                    for (uint32_t j = 0; j < n; ++j) {
                        const uint32_t m = (uint32_t)(keys[j] & 0xFFFFFFFFull);
                        if (pass == 0) warmStartOne(a, j, m);
                        else solveOneChained(a, j, m);
                    }
            }
            __syncwarp();
            continue;
        }
        const uint32_t r = i < nFront ? queue[i] : queue[nIsl - 1 - (i - nFront)];
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

// Large islands, all together: bucket their manifolds by colour (the
// bucket lists live in islKeysTmp), then warm start and iterations colour by
// colour with a grid barrier after each colour.  Every block reads the same
// counts, so with no large island all return before the first barrier.
// More than kMaxColors colours: every island in grid-wide sweeps, the
// per-colour counts in sb.colorStart scanned into starts by block 0, then used
// as fill cursors (after the fill, colorStart[c] is the end of colour c).
__device__ void islSolveWide(const SolveArgs &a, uint32_t M, uint32_t C) {
    __shared__ uint32_t s_scan[9], s_carry;
    uint32_t *cur = a.sb.colorStart;
    if (blockIdx.x == 0) {
        if (threadIdx.x == 0) s_carry = 0;
        __syncthreads();
        for (uint32_t c0 = 0; c0 < C; c0 += blockDim.x) {
            const uint32_t c = c0 + threadIdx.x;
            const uint32_t v = c < C ? __ldcg(&cur[c]) : 0u;
            uint32_t total;
            const uint32_t ex = blockExclusiveScan(v, total, s_scan);
            if (c < C) __stcg(&cur[c], s_carry + ex);
            __syncthreads();
            if (threadIdx.x == 0) s_carry += total;
            __syncthreads();
        }
    }
    if (!gridBarrier(a.sb.bar, &a.st->err)) return;
    const uint32_t *cnt = islCnt(a);
    uint32_t *list = reinterpret_cast<uint32_t *>(a.sb.islKeysTmp);
    const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, gstride = gridDim.x * blockDim.x;
    for (uint32_t m = gtid; m < M; m += gstride) {
        const uint32_t r = a.sb.islRoot[m];
        const uint32_t c = a.sb.color[m];
        if (r == kIslNone || cnt[r] == 0 || c >= C) continue;
        list[aggregatedAppendKeyed(cur, c)] = m;
    }
    if (!gridBarrier(a.sb.bar, &a.st->err)) return;
    for (int pass = 0; pass <= a.iterations; ++pass)
        for (uint32_t c = 0; c < C; ++c) {
            const uint32_t lo = c ? __ldcg(&cur[c - 1]) : 0u, hi = __ldcg(&cur[c]);
            for (uint32_t k = lo + gtid; k < hi; k += gstride) {
                if (pass == 0) warmStartOne(a, k, list[k]);
                else solveOne(a, k, list[k]);
            }
            if (!gridBarrier(a.sb.bar, &a.st->err)) return;
        }
}

// GlobalVel with the manifold's bodies already loaded.
struct BodiesGiven {
    const SolveArgs &a;
    uint2 b;
    __device__ __forceinline__ uint2 bodies(uint32_t, uint32_t) const { return b; }
    __device__ __forceinline__ V3 lin(uint32_t i) const { return f4xyz(ld4(&a.w.nxt.lin[i])); }
    __device__ __forceinline__ V3 ang(uint32_t i) const { return f4xyz(ld4(&a.w.nxt.ang[i])); }
    __device__ __forceinline__ void store(uint32_t i, const V3 &l, const V3 &w) const {
        st4(&a.w.nxt.lin[i], make4(l, 0.0f));
        st4(&a.w.nxt.ang[i], make4(w, 0.0f));
    }
};

// Grid-wide sweeps: each thread keeps one shared-memory slot holding the
// prepared data of its manifold of the coming colour step (the manifold's
// normal and masses, then per point the ten prepared vectors and the
// impulse), laid out field-major across the block's threads.  The copy is
// issued (cp.async) as soon as the thread has finished its manifold of the
// current step, so it lands while the grid waits at the colour barrier; after
// the barrier only the body velocities are loaded from memory.
constexpr uint32_t kSlotPoint = kPreparedVec4 + 1;                 // prepared vectors + impulse
constexpr uint32_t kSlotVec4 = 2 + 4 * kSlotPoint;                 // pm, pn, 4 points
constexpr size_t kLargeSmem = (size_t)kSlotVec4 * kSolveThreads * sizeof(float4);  // 188,416 bytes
// List entries of the grid-wide sweeps: manifold index | solved points << 29.
constexpr uint32_t kEntryShift = 29;
constexpr uint32_t kEntryMask = (1u << kEntryShift) - 1u;

__device__ __forceinline__ void cpAsync16(float4 *dst, const float4 *src) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cpAsyncCommit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cpAsyncWaitAll() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// slot: this thread's column (s_slot + threadIdx.x), stride kSolveThreads.
__device__ __forceinline__ void fetchSlot(const SolveArgs &a, float4 *slot, uint32_t m, uint32_t npts) {
    const uint32_t mcap = a.mcap;
    cpAsync16(slot, &a.sb.pm[m]);
    cpAsync16(slot + kSolveThreads, &a.sb.pn[m]);
    for (uint32_t p = 0; p < npts; ++p) {
        float4 *d = slot + (size_t)(2 + p * kSlotPoint) * kSolveThreads;
#pragma unroll
        for (uint32_t v = 0; v < (uint32_t)kPreparedVec4; ++v)
            cpAsync16(d + (size_t)v * kSolveThreads, &a.sb.pp[(size_t)(v * 4 + p) * mcap + m]);
        cpAsync16(d + (size_t)kPreparedVec4 * kSolveThreads, &a.sb.pimp[(size_t)p * mcap + m]);
    }
    cpAsyncCommit();
}

// Prepared data of one manifold from this thread's slot; impulses are written
// back to the solver arrays (the slot is refilled for every colour step).
struct SlotPrep {
    const SolveArgs &a;
    const float4 *slot;
    uint32_t m, npts;
    __device__ __forceinline__ float4 pm(uint32_t) const { return slot[0]; }
    __device__ __forceinline__ float4 pn(uint32_t) const { return slot[kSolveThreads]; }
    __device__ __forceinline__ uint32_t count(uint32_t) const { return npts; }
    __device__ __forceinline__ float4 inertia(int r, uint32_t) const {
        return a.sb.pmInertia[(size_t)r * a.mcap + m];
    }
    __device__ __forceinline__ float4 pt(int v, uint32_t p, uint32_t) const {
        return slot[(size_t)(2 + p * kSlotPoint + v) * kSolveThreads];
    }
    __device__ __forceinline__ float4 imp(uint32_t p, uint32_t) const {
        return slot[(size_t)(2 + p * kSlotPoint + kPreparedVec4) * kSolveThreads];
    }
    __device__ __forceinline__ void setImp(uint32_t p, uint32_t, const float4 &v) const {
        a.sb.pimp[(size_t)p * a.mcap + m] = v;
    }
};

__global__ void __launch_bounds__(kSolveThreads) k_isl_solve_large(SolveArgs a) {
    __shared__ uint32_t s_start[kMaxColors + 1];
    __shared__ uint32_t s_colors[kMaxColors], s_colorN;
    extern __shared__ float4 s_slot[];
    {
        const uint32_t M = min(*a.count, a.mcap);
        const uint32_t wideC = islWideColors(a, M);
        if (wideC) {  // every block sees the same colour count
            islSolveWide(a, M, wideC);
            return;
        }
    }
    const uint32_t *count = a.sb.islCounters + kIslColorCount;
    uint32_t *fill = a.sb.islCounters + kIslColorFill;
    if (threadIdx.x == 0) {
        uint32_t acc = 0;
        for (int c = 0; c < kMaxColors; ++c) {
            s_start[c] = acc;
            acc += count[c];
        }
        s_start[kMaxColors] = acc;
    }
    __syncthreads();
    if (s_start[kMaxColors] == 0) return;
    const uint32_t M = min(*a.count, a.mcap);
    const uint32_t *cnt = islCnt(a);
    const uint32_t sweepFrom = islSweepFrom(a, M);
    uint32_t *list = reinterpret_cast<uint32_t *>(a.sb.islKeysTmp);
    const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, gstride = gridDim.x * blockDim.x;
    for (uint32_t m = gtid; m < M; m += gstride) {
        const uint32_t r = a.sb.islRoot[m];
        const uint32_t c = a.sb.color[m];
        if (r == kIslNone || cnt[r] < sweepFrom || c >= (uint32_t)kMaxColors) continue;
        list[s_start[c] + aggregatedAppendKeyed(fill, c)] = m | min(a.sb.pcount[m], 4u) << kEntryShift;
    }
    // the non-empty colours, in order
    if (threadIdx.x == 0) {
        uint32_t n = 0;
        for (int c = 0; c < kMaxColors; ++c)
            if (s_start[c] != s_start[c + 1]) s_colors[n++] = (uint32_t)c;
        s_colorN = n;
    }
    if (!gridBarrier(a.sb.bar, &a.st->err)) return;
    // Colour steps in (pass, colour) order.  A thread's first manifold of a
    // step is the same in every pass.  Its
    // list entry is loaded while the step before is solved, its bodies and
    // (passes after the warm start) its slot right after that step, before
    // the barrier; further manifolds of the step (more than one per thread)
    // read the solver arrays.
    // Solve index j of a colour goes to block j % gridDim.x, thread j /
    // gridDim.x: a colour's manifolds are spread over every SM of the grid
    // (a thin colour keeps one warp per block busy, not a few full blocks).
    const uint32_t nC = s_colorN;
    const uint32_t nSteps = nC * (uint32_t)(a.iterations + 1);
    const uint32_t lane = threadIdx.x * gridDim.x + blockIdx.x;
    float4 *slot = s_slot + threadIdx.x;
    const GlobalPrep gp{a};
    auto firstIndex = [&](uint32_t step) { return s_start[s_colors[step % nC]] + lane; };
    auto stepEnd = [&](uint32_t step) { return s_start[s_colors[step % nC] + 1]; };
    uint32_t e = 0;
    uint2 b = make_uint2(0u, 0u);
    if (firstIndex(0) < stepEnd(0)) {
        e = __ldcg(&list[firstIndex(0)]);
        b = __ldcg(&a.sb.pbody[e & kEntryMask]);
    }
    for (uint32_t step = 0; step < nSteps; ++step) {
        const uint32_t pass = step / nC;
        const uint32_t k0 = firstIndex(step), end = stepEnd(step);
        const bool next = step + 1 < nSteps && firstIndex(step + 1) < stepEnd(step + 1);
        const uint32_t eNext = next ? __ldcg(&list[firstIndex(step + 1)]) : 0u;
        if (k0 < end) {
            const uint32_t m = e & kEntryMask;
            const BodiesGiven v{a, b};
            if (pass == 0) {
                warmStartOne(gp, k0, m, v);
            } else {
                cpAsyncWaitAll();
                solveOne(SlotPrep{a, slot, m, e >> kEntryShift}, k0, m, v);
            }
            for (uint32_t k = k0 + gstride; k < end; k += gstride) {
                const uint32_t mk = __ldcg(&list[k]) & kEntryMask;
                const BodiesGiven vk{a, __ldcg(&a.sb.pbody[mk])};
                if (pass == 0) warmStartOne(gp, k, mk, vk);
                else solveOneChained(gp, k, mk, vk);
            }
        }
        if (next) {
            e = eNext;
            b = __ldcg(&a.sb.pbody[e & kEntryMask]);
            if ((step + 1) / nC > 0) fetchSlot(a, slot, e & kEntryMask, e >> kEntryShift);
        }
        if (!gridBarrier(a.sb.bar, &a.st->err)) {
            cpAsyncWaitAll();  // no copy into shared memory outlives the block
            return;
        }
    }
    cpAsyncWaitAll();
}

namespace {
void configureLargeSweeps() {
    static bool configured = false;
    if (!configured) {
        PE_CHECK(cudaFuncSetAttribute(k_isl_solve_large, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kLargeSmem));
        configured = true;
    }
}
} // namespace

int solveIslandsBlocksPerSm() {
    configureLargeSweeps();
    int b = 0;
    PE_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_isl_solve_large, kSolveThreads, kLargeSmem));
    return b;
}

void launchSolveIslands(const SolveArgs &a, int coopBlocks, Scratch &ws, cudaStream_t s) {
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
    k_isl_solve<<<4 * smCount(), kIslThreads, 0, s>>>(a);
    PE_LAUNCHED();
    // list entries carry the manifold index in kEntryShift bits
    if (mcap > kEntryMask) throw std::length_error("manifold capacity beyond the grid-wide sweeps' index range");
    configureLargeSweeps();
    SolveArgs args = a;
    void *params[] = {&args};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(coopBlocks);
    cfg.blockDim = dim3(kSolveThreads);
    cfg.dynamicSmemBytes = kLargeSmem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    PE_CHECK(cudaLaunchKernelExC(&cfg, (const void *)k_isl_solve_large, params));
    PE_LAUNCHED();
}

void setSpinLimitIslands(uint32_t limit) { setSpinLimitOfUnit(limit); }

} // namespace pe
