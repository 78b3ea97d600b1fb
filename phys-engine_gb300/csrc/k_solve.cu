// Contact solver: graph-coloured projected Gauss-Seidel.
//
// The reference solves manifolds one after another
// (src/solver/sequential_impulse_solver.cpp:226-684).  Here manifolds are
// coloured so that no two manifolds of one colour share a non-static body, and
// the sequential sweep is run colour by colour with all manifolds of a colour in
// parallel.  Static bodies are never written (the reference's apply lambdas
// return early for them, :288-310), so this equals the reference fed the
// manifolds in (colour, index) order, bit for bit.
//
// Colouring: priority(m) = a bijective 32-bit mix of m; every manifold takes the
// smallest colour not used by a higher-priority manifold sharing one of its
// dynamic bodies (greedy in decreasing priority).  Computed without rounds: each
// body lists its manifolds (up to kIslandMax), and a manifold is coloured as soon
// as every higher-priority manifold at its dynamic bodies has its colour — the
// colour then depends on those colours only, whenever it is computed.  A body
// with more manifolds sends the step to parallel rounds (Jones-Plassmann): a
// manifold is coloured once it holds the highest priority among the uncoloured
// manifolds at both its bodies; the same colouring.
#include "pe_block.cuh"
#include "pe_kernels.cuh"
#include "pe_solve.cuh"
#include "pe_stages.h"

namespace pe {

// ------------------------------------------------------------- colouring ---
// Manifolds per thread whose higher-priority neighbours the colouring keeps
// in shared memory (32 slots each: two bodies x kIslandMax list entries).
constexpr uint32_t kColorCached = 6;
constexpr uint32_t kColorSlots = 2 * kIslandMax;
constexpr uint32_t kNoNeighbour = 0xFFFFFFFFu;
constexpr size_t kColorSmem = (size_t)kColorCached * kColorSlots * kSolveThreads * sizeof(uint32_t);  // 196,608 bytes

__global__ void __launch_bounds__(kSolveThreads) k_color(SolveArgs a) {
    extern __shared__ uint32_t s_hp[];  // [kColorCached][kColorSlots][blockDim.x]
    const uint32_t M = min(*a.count, a.mcap);
    const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, gstride = gridDim.x * blockDim.x;
    const WorldView &w = a.w;
    SolverBuffers &sb = a.sb;
    // per-body manifold lists: counts in islOff, lists in islandList (both
    // free until the island sweeps)
    uint32_t *incCount = sb.islOff, *inc = sb.islandList;
    if (M == 0) {  // nothing to colour (every block sees the same count)
        if (blockIdx.x == 0)
            for (int c = threadIdx.x; c < kMaxColors; c += blockDim.x) sb.colorCount[c] = 0;
        return;
    }
    for (uint32_t m = gtid; m < M; m += gstride) {
        uint32_t ba = a.mv.bodyA[m], bb = a.mv.bodyB[m];
        bool da = ba < w.nb && w.bgen[ba] == a.mv.genA[m] && bodyMoves(w.bflags[ba]);
        bool db = bb < w.nb && w.bgen[bb] == a.mv.genB[m] && bodyMoves(w.bflags[bb]);
        sb.dyn[m] = (da ? 1u : 0u) | (db ? 2u : 0u);
        sb.color[m] = kUncolored;
        if (da) {
            __stcg(&sb.bodyUsed[2 * ba], 0ull);
            __stcg(&sb.bodyUsed[2 * ba + 1], 0ull);
            __stcg(&incCount[ba], 0u);
        }
        if (db) {
            __stcg(&sb.bodyUsed[2 * bb], 0ull);
            __stcg(&sb.bodyUsed[2 * bb + 1], 0ull);
            __stcg(&incCount[bb], 0u);
        }
    }
    if (blockIdx.x == 0)
        for (int c = threadIdx.x; c < kMaxColors; c += blockDim.x) sb.colorCount[c] = 0;
    if (!gridBarrier(sb.bar, &a.st->err)) return;
    // each dynamic body's manifolds
    for (uint32_t m = gtid; m < M; m += gstride) {
        const uint32_t d = sb.dyn[m];
        for (int e = 0; e < 2; ++e) {
            if (!(d & (1u << e))) continue;
            const uint32_t b = e ? a.mv.bodyB[m] : a.mv.bodyA[m];
            const uint32_t slot = atomicAdd(&incCount[b], 1u);
            if (slot < kIslandMax) inc[(size_t)b * kIslandMax + slot] = m;
            else sb.counters[1] = 1u;
        }
    }
    if (!gridBarrier(sb.bar, &a.st->err)) return;
    if (__ldcg(&sb.counters[1]) == 0u && (M + gstride - 1) / gstride <= kColorCached) {
        // Each thread reads its manifolds' neighbour lists once and keeps the
        // higher-priority neighbours in shared memory; every pass then asks
        // for all of a manifold's neighbour colours in one round trip.
        const uint32_t T = blockDim.x, R = (M + gstride - 1) / gstride;
        uint32_t pendingMask = 0;
        for (uint32_t k = 0; k < R; ++k) {
            const uint32_t m = gtid + k * gstride;
            if (m >= M) continue;
            pendingMask |= 1u << k;
            uint32_t *row = s_hp + (size_t)k * kColorSlots * T + threadIdx.x;
            const uint32_t p = colorPriority(m), d = sb.dyn[m];
            uint32_t n[2], bs[2];
            for (int e = 0; e < 2; ++e) {
                bs[e] = e ? a.mv.bodyB[m] : a.mv.bodyA[m];
                n[e] = (d & (1u << e)) ? min(__ldcg(&incCount[bs[e]]), kIslandMax) : 0u;
            }
            uint32_t o[kColorSlots];
#pragma unroll
            for (uint32_t i = 0; i < kColorSlots; ++i) {
                const uint32_t e = i / kIslandMax, j = i % kIslandMax;
                o[i] = j < n[e] ? __ldcg(&inc[(size_t)bs[e] * kIslandMax + j]) : kNoNeighbour;
            }
#pragma unroll
            for (uint32_t i = 0; i < kColorSlots; ++i)
                row[(size_t)i * T] = (o[i] != kNoNeighbour && o[i] != m && colorPriority(o[i]) > p) ? o[i]
                                                                                                  : kNoNeighbour;
        }
        uint32_t pass = 0;
        for (; pendingMask && pass < spinLimit(); ++pass) {
            for (uint32_t k = 0; k < R; ++k) {
                if (!(pendingMask >> k & 1u)) continue;
                const uint32_t m = gtid + k * gstride;
                const uint32_t *row = s_hp + (size_t)k * kColorSlots * T + threadIdx.x;
                uint32_t cs[kColorSlots];
#pragma unroll
                for (uint32_t i = 0; i < kColorSlots; ++i) {
                    const uint32_t o = row[(size_t)i * T];
                    cs[i] = o != kNoNeighbour ? ldvol(&sb.color[o]) : 0xFFFFFFFEu;
                }
                unsigned long long u0 = 0, u1 = 0;
                bool ready = true;
#pragma unroll
                for (uint32_t i = 0; i < kColorSlots; ++i) {
                    if (cs[i] == 0xFFFFFFFEu) continue;
                    if (cs[i] == kUncolored) ready = false;
                    else if (cs[i] < 64) u0 |= 1ull << cs[i];
                    else u1 |= 1ull << (cs[i] - 64);
                }
                if (!ready) continue;
                uint32_t c;
                if (~u0) c = __ffsll((long long)~u0) - 1;
                else if (~u1) c = 64 + __ffsll((long long)~u1) - 1;
                else {
                    atomicOr(&a.st->err, kErrColors);
                    c = kMaxColors - 1;
                }
                *(volatile uint32_t *)&sb.color[m] = c;
                aggregatedAppendKeyed(sb.colorCount, c);
                aggregatedMax32(&a.st->colors, c + 1);
                pendingMask &= ~(1u << k);
            }
        }
        if (pendingMask) atomicOr(&a.st->err, kErrTimeout);
        aggregatedMax32(&a.st->colorRounds, pass);
        return;
    }
    if (__ldcg(&sb.counters[1]) == 0u) {
        uint32_t pass = 0;
        bool pending = true;
        for (; pending && pass < spinLimit(); ++pass) {
            pending = false;
            for (uint32_t m = gtid; m < M; m += gstride) {
                if (sb.color[m] != kUncolored) continue;
                const uint32_t p = colorPriority(m), d = sb.dyn[m];
                unsigned long long u0 = 0, u1 = 0;
                bool ready = true;
                for (int e = 0; e < 2 && ready; ++e) {
                    if (!(d & (1u << e))) continue;
                    const uint32_t b = e ? a.mv.bodyB[m] : a.mv.bodyA[m];
                    const uint32_t n = min(__ldcg(&incCount[b]), kIslandMax);
                    const uint32_t *list = inc + (size_t)b * kIslandMax;
                    uint32_t cs[kIslandMax];
#pragma unroll
                    for (uint32_t i = 0; i < kIslandMax; ++i) {
                        cs[i] = 0xFFFFFFFEu;  // not a higher-priority neighbour
                        if (i < n) {
                            const uint32_t o = __ldcg(&list[i]);
                            if (o != m && colorPriority(o) > p) cs[i] = ldvol(&sb.color[o]);
                        }
                    }
#pragma unroll
                    for (uint32_t i = 0; i < kIslandMax; ++i) {
                        if (cs[i] == 0xFFFFFFFEu) continue;
                        if (cs[i] == kUncolored) ready = false;
                        else if (cs[i] < 64) u0 |= 1ull << cs[i];
                        else u1 |= 1ull << (cs[i] - 64);
                    }
                }
                if (!ready) {
                    pending = true;
                    continue;
                }
                uint32_t c;
                if (~u0) c = __ffsll((long long)~u0) - 1;
                else if (~u1) c = 64 + __ffsll((long long)~u1) - 1;
                else {
                    atomicOr(&a.st->err, kErrColors);
                    c = kMaxColors - 1;
                }
                *(volatile uint32_t *)&sb.color[m] = c;
                aggregatedAppendKeyed(sb.colorCount, c);
                aggregatedMax32(&a.st->colors, c + 1);
            }
        }
        if (pending) atomicOr(&a.st->err, kErrTimeout);
        aggregatedMax32(&a.st->colorRounds, pass);
        return;
    }
    // Jones-Plassmann rounds in colour windows of kMaxColors (see kDeferred):
    // counters[0] counts manifolds done in the window (coloured or deferred),
    // counters[2] the deferred ones.
    const unsigned long long epoch0 = __ldcg(sb.epoch);
    uint32_t rounds = 0, base = 0;
    bool exhausted = false;
    for (;;) {
        uint32_t round = 0;
        for (; round < kMaxRounds; ++round) {
            const unsigned long long stamp = (epoch0 + rounds + round + 1) << 32;
            for (uint32_t m = gtid; m < M; m += gstride) {
                if (sb.color[m] != kUncolored) continue;
                const unsigned long long p = stamp | colorPriority(m);
                const uint32_t d = sb.dyn[m];
                if (d & 1u) atomicMax(&sb.bodyBest[a.mv.bodyA[m]], p);
                if (d & 2u) atomicMax(&sb.bodyBest[a.mv.bodyB[m]], p);
            }
            if (!gridBarrier(sb.bar, &a.st->err)) return;
            for (uint32_t m = gtid; m < M; m += gstride) {
                if (sb.color[m] != kUncolored) continue;
                const unsigned long long p = stamp | colorPriority(m);
                const uint32_t d = sb.dyn[m];
                const uint32_t ba = a.mv.bodyA[m], bb = a.mv.bodyB[m];
                if ((d & 1u) && __ldcg(&sb.bodyBest[ba]) != p) continue;
                if ((d & 2u) && __ldcg(&sb.bodyBest[bb]) != p) continue;
                unsigned long long u0 = 0, u1 = 0;
                if (d & 1u) {
                    u0 |= __ldcg(&sb.bodyUsed[2 * ba]);
                    u1 |= __ldcg(&sb.bodyUsed[2 * ba + 1]);
                }
                if (d & 2u) {
                    u0 |= __ldcg(&sb.bodyUsed[2 * bb]);
                    u1 |= __ldcg(&sb.bodyUsed[2 * bb + 1]);
                }
                uint32_t local = kDeferred;
                if (~u0) local = __ffsll((long long)~u0) - 1;
                else if (~u1) local = 64 + __ffsll((long long)~u1) - 1;
                if (local == kDeferred) {
                    sb.color[m] = kDeferred;
                    aggregatedAppend(&sb.counters[2]);
                } else {
                    const uint32_t c = base + local;
                    sb.color[m] = c;
                    const unsigned long long bit = 1ull << (local & 63);
                    const uint32_t word = local >> 6;
                    if (d & 1u) __stcg(&sb.bodyUsed[2 * ba + word], __ldcg(&sb.bodyUsed[2 * ba + word]) | bit);
                    if (d & 2u) __stcg(&sb.bodyUsed[2 * bb + word], __ldcg(&sb.bodyUsed[2 * bb + word]) | bit);
                    if (c < (uint32_t)kMaxColors) aggregatedAppendKeyed(sb.colorCount, c);
                    aggregatedMax32(&a.st->colors, c + 1);
                }
                aggregatedAppend(&sb.counters[0]);
            }
            if (!gridBarrier(sb.bar, &a.st->err)) return;
            if (__ldcg(&sb.counters[0]) >= M) break;
        }
        rounds += round + 1;
        if (round >= kMaxRounds) {
            exhausted = true;
            break;
        }
        const uint32_t deferred = __ldcg(&sb.counters[2]);
        if (deferred == 0) break;
        // next window: deferred manifolds uncoloured again, their bodies'
        // masks empty
        base += kMaxColors;
        for (uint32_t m = gtid; m < M; m += gstride) {
            if (sb.color[m] != kDeferred) continue;
            sb.color[m] = kUncolored;
            const uint32_t d = sb.dyn[m];
            if (d & 1u) {
                __stcg(&sb.bodyUsed[2 * a.mv.bodyA[m]], 0ull);
                __stcg(&sb.bodyUsed[2 * a.mv.bodyA[m] + 1], 0ull);
            }
            if (d & 2u) {
                __stcg(&sb.bodyUsed[2 * a.mv.bodyB[m]], 0ull);
                __stcg(&sb.bodyUsed[2 * a.mv.bodyB[m] + 1], 0ull);
            }
        }
        if (!gridBarrier(sb.bar, &a.st->err)) return;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            sb.counters[0] = M - deferred;
            sb.counters[2] = 0;
        }
        if (!gridBarrier(sb.bar, &a.st->err)) return;
    }
    if (exhausted) {
        // The step fails (kErrColors); colour 0 for what is left keeps every
        // colour index in range.
        for (uint32_t m = gtid; m < M; m += gstride)
            if (sb.color[m] >= kDeferred) sb.color[m] = 0;
        aggregatedMax32(&a.st->colors, 1u);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *sb.epoch = epoch0 + rounds + 2;
        a.st->colorRounds = rounds;
        if (exhausted) atomicOr(&a.st->err, kErrColors);
    }
}

// With sleeping on: the solver takes every manifold while some body is awake,
// none otherwise (a contact among static and sleeping bodies is not solved).
__global__ void k_solve_count(DevStats *st) {
    if (threadIdx.x == 0) st->solveCount = st->awakeInStep ? st->manifolds : 0u;
}

__global__ void k_order_init(SolveArgs a, int serial) {
    const uint32_t M = min(*a.count, a.mcap);
    for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
        a.sb.orderKeys[m] = serial ? 0u : a.sb.color[m];
        a.sb.order[m] = m;
    }
}

// Prepare of every manifold, by manifold index, before the colouring, and the
// manifold flags (sb.dyn) the single-block front reads.  The old cache's keys
// are copied to shared memory when at most keyCap of them.
constexpr int kPrepareThreads = 64;
constexpr uint32_t kPrepareKeyCap = 4096;
__global__ void __launch_bounds__(kPrepareThreads) k_prepare(SolveArgs a, uint32_t keyCap) {
    extern __shared__ unsigned long long s_keys[];
    const uint32_t M = min(*a.count, a.mcap);
    for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x)
        a.sb.dyn[m] = manifoldFlags(a, m);
    const uint32_t cacheN = *a.oldCount;
    const bool inShared = cacheN <= keyCap;
    if (inShared)
        for (uint32_t i = threadIdx.x; i < cacheN; i += blockDim.x) s_keys[i] = a.oldCache.key[i];
    __syncthreads();
    prepareRange(a, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, min(*a.count, a.mcap),
                 inShared ? s_keys : nullptr);
}

// Manifold order (the reference's own sequence), one thread.
__global__ void k_solve_serial(SolveArgs a) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const uint32_t M = min(*a.count, a.mcap);
    for (uint32_t k = 0; k < M; ++k) warmStartOne(a, k, k);
    for (int it = 0; it < a.iterations; ++it)
        for (uint32_t k = 0; k < M; ++k) solveOne(a, k, k);
}

// Solved impulses of the live points back to the manifolds (pair order).
__global__ void k_impulses_out(SolveArgs a) {
    const uint32_t M = min(*a.count, a.mcap);
    for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
        const uint32_t live = a.sb.pcount[m];
        for (uint32_t p = 0; p < live; ++p) {
            float4 imp = a.sb.pimp[(size_t)p * a.mcap + m];
            imp.w = 0.0f;
            a.mv.impulse[4 * m + p] = imp;
        }
    }
}

// ---------------------------------------------------------- cache rebuild --
// Next cache (:623-681): every point of every solved manifold, sorted by body
// pair, stable with respect to solve order.
// Sort key (bodyA << bits) | bodyB: the (bodyA, bodyB) order of the cache.
__global__ void k_cache_keys(SolveArgs a, uint32_t bits) {
    const uint32_t M = min(*a.count, a.mcap);
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < M; k += gridDim.x * blockDim.x) {
        const uint32_t m = a.sb.order[k];
        a.sb.cacheKeys[k] = ((unsigned long long)a.mv.bodyA[m] << bits) | a.mv.bodyB[m];
        a.sb.cacheVals[k] = m;
    }
}
__global__ void k_cache_counts(SolveArgs a) {
    const uint32_t M = min(*a.count, a.mcap);
    const WorldView &w = a.w;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < M; k += gridDim.x * blockDim.x) {
        const uint32_t m = a.pairOrderCache ? k : a.sb.cacheVals[k];
        const uint32_t ia = a.mv.bodyA[m], ib = a.mv.bodyB[m];
        const bool valid = ia < w.nb && ib < w.nb && (w.bflags[ia] & kBodyAlive) && (w.bflags[ib] & kBodyAlive) &&
                           w.bgen[ia] == a.mv.genA[m] && w.bgen[ib] == a.mv.genB[m] &&
                           solvedPair(w, w.bflags[ia], w.bflags[ib]);
        a.sb.cacheCounts[k] = valid ? min(a.mv.pointCount[m], 4u) : 0u;
    }
}
// Writes the cache entries of manifold m (npts points) starting at entry base.
__global__ void k_cache_write(SolveArgs a, CacheView nc, uint32_t cacheCap) {
    const uint32_t M = min(*a.count, a.mcap);
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < M; k += gridDim.x * blockDim.x)
        cacheWriteManifold(a, nc, cacheCap, a.pairOrderCache ? k : a.sb.cacheVals[k], a.sb.cacheOff[k],
                           a.sb.cacheCounts[k]);
}


// Velocity staging slots of the single-block solver (bodies touched by contacts).
constexpr uint32_t kStageSlots = 3072;
constexpr size_t blockSolveSmem(uint32_t blockM, uint32_t stageSlots) {
    return (size_t)blockM * (8 + 4 + 8) + (size_t)stageSlots * (32 + 4);
}

// blockM: manifold capacity of this launch (power of two); shared memory is
// sized for it and for `stageSlots` staged bodies, so that the rest of the
// SM's unified L1 / shared storage caches the prepared contact constants.
__global__ void __launch_bounds__(kBlockSolveThreads)
k_solve_block(SolveArgs a, CacheView nc, uint32_t cacheCap, uint32_t *newCount, int serial, uint32_t blockM,
              uint32_t stageSlots) {
    // The manifolds were prepared by k_prepare, launched before this kernel.
    // blockM u64 sort keys, u32 flags, uint2 stage slots; then the staged
    // velocities (2 float4 per slot) and the body of each slot.
    extern __shared__ unsigned long long s_sort[];
    __shared__ BlockSolveShared sh;
    unsigned char *base = reinterpret_cast<unsigned char *>(s_sort);
    VelStage vs;
    vs.slot = reinterpret_cast<uint2 *>(base + (size_t)blockM * 12);
    vs.v = reinterpret_cast<float4 *>(base + (size_t)blockM * 20);
    vs.slotBody = reinterpret_cast<uint32_t *>(base + (size_t)blockM * 20 + (size_t)stageSlots * 32);
    vs.cap = stageSlots;
    solveBlock(a, nc, cacheCap, newCount, serial, blockM, s_sort, reinterpret_cast<uint32_t *>(s_sort + blockM), sh,
               stageSlots ? &vs : nullptr, true);
}

static int gridFor(uint32_t n, int threads = 256, int maxBlocks = 0) {
    if (maxBlocks <= 0) maxBlocks = 8 * smCount();
    uint32_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    return (int)(b < (uint32_t)maxBlocks ? b : (uint32_t)maxBlocks);
}

static void launchCooperative(const void *fn, int blocks, SolveArgs &args, cudaStream_t s, size_t smem = 0) {
    void *params[] = {&args};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(kSolveThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    PE_CHECK(cudaLaunchKernelExC(&cfg, fn, params));
    ++g_kernelLaunches;
}

static void configureColor() {
    static bool configured = false;
    if (!configured) {
        PE_CHECK(cudaFuncSetAttribute(k_color, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kColorSmem));
        configured = true;
    }
}

int maxCooperativeBlocks(int smCount) {
    static int perSm = -1;
    if (perSm < 0) {
        configureColor();
        int a = 0;
        PE_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_color, kSolveThreads, kColorSmem));
        const int b = solveIslandsBlocksPerSm();
        perSm = a < b ? a : b;
        if (perSm < 1) perSm = 1;
    }
    return perSm * smCount;
}

void launchSolver(const WorldView &w, const ManifoldView &mv, const CacheView &oldCache, const uint32_t *oldCacheCount,
                  const CacheView &newCache, uint32_t *newCacheCount, uint32_t cacheCap, SolverBuffers &sb,
                  int iterations, int orderMode, int coopBlocks, bool blockPath, uint32_t blockM, bool pairOrderCache,
                  DevStats *st, Scratch &ws, cudaStream_t s) {
    SolveArgs a{w, mv, sb, oldCache, oldCacheCount, st, sb.mcap, iterations, pairOrderCache,
                w.sleepMode ? &st->solveCount : &st->manifolds};
    if (w.sleepMode) {
        k_solve_count<<<1, 32, 0, s>>>(st);
        PE_LAUNCHED();
    }
    uint32_t *err = &st->err;
    const uint32_t mcap = sb.mcap;
    if (blockPath) {
        static bool configured = false;
        if (!configured) {
            PE_CHECK(cudaFuncSetAttribute(k_solve_block, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)blockSolveSmem(kBlockMaxManifolds, kStageSlots)));
            configured = true;
        }
        uint32_t bm = kBlockMaxManifolds;
        if (blockM && blockM < kBlockMaxManifolds) {
            bm = 64;
            while (bm < blockM) bm <<= 1;
        }
        uint32_t slots = 2 * bm < kStageSlots ? 2 * bm : kStageSlots;
        if (orderMode != 0 && launchSolverCluster(a, newCache, newCacheCount, cacheCap, bm, slots, s)) return;
        const size_t smem = blockSolveSmem(bm, slots);
        k_prepare<<<(4 * bm + kPrepareThreads - 1) / kPrepareThreads, kPrepareThreads,
                    kPrepareKeyCap * sizeof(unsigned long long), s>>>(a, kPrepareKeyCap);
        PE_LAUNCHED();
        k_solve_block<<<1, kBlockSolveThreads, smem, s>>>(a, newCache, cacheCap, newCacheCount, orderMode == 0 ? 1 : 0,
                                                          bm, slots);
        PE_LAUNCHED();
        return;
    }
    PE_CHECK(cudaMemsetAsync(sb.counters, 0, 4 * sizeof(uint32_t), s));
    PE_CHECK(cudaMemsetAsync(sb.bar, 0, 2 * sizeof(uint32_t), s));
    const bool serial = orderMode == 0;
    if (!serial) {
        configureColor();
        launchCooperative((const void *)k_color, coopBlocks, a, s, kColorSmem);
    }
    // the solve order itself is needed by the serial sweep and by a cache
    // rebuilt in solve order; the island sweeps order each island themselves
    if (serial || !pairOrderCache) {
        k_order_init<<<gridFor(mcap), 256, 0, s>>>(a, serial ? 1 : 0);
        PE_LAUNCHED();
        // colours may exceed 255 (colour windows); passes over constant
        // digits are skipped on the device
        if (!serial)
            launchRadixSort<uint32_t>(sb.orderKeys, sb.orderKeysTmp, sb.order, sb.orderTmp, a.count, mcap, 0, 32,
                                      ws, err, s);
    }
    k_prepare<<<gridFor(mcap, kPrepareThreads), kPrepareThreads, kPrepareKeyCap * sizeof(unsigned long long), s>>>(
        a, kPrepareKeyCap);
    PE_LAUNCHED();
    if (serial) {
        k_solve_serial<<<1, 32, 0, s>>>(a);
        PE_LAUNCHED();
    } else {
        launchSolveIslands(a, coopBlocks, ws, s);
    }
    k_impulses_out<<<gridFor(mcap), 256, 0, s>>>(a);
    PE_LAUNCHED();
    if (!pairOrderCache) {
        // several manifolds may share a body pair: cache order = (body pair,
        // solve order), a stable sort of the solve order by pair key
        uint32_t keyBits = 1;
        while (keyBits < 32 && (1ull << keyBits) < (unsigned long long)(w.nb > 2 ? w.nb : 2)) ++keyBits;
        k_cache_keys<<<gridFor(mcap), 256, 0, s>>>(a, keyBits);
        PE_LAUNCHED();
        launchRadixSort<unsigned long long>(sb.cacheKeys, sb.cacheKeysTmp, sb.cacheVals, sb.cacheValsTmp,
                                            a.count, mcap, 0, 2 * (int)keyBits, ws, err, s);
    }
    // else one manifold per body pair, in (body A, body B) order: the cache is
    // the manifolds' points in manifold order
    k_cache_counts<<<gridFor(mcap), 256, 0, s>>>(a);
    PE_LAUNCHED();
    launchScanExclusive(sb.cacheCounts, sb.cacheOff, a.count, mcap, newCacheCount, ws, err, s);
    k_cache_write<<<gridFor(mcap), 256, 0, s>>>(a, newCache, cacheCap);
    PE_LAUNCHED();
}

void setSpinLimitSolve(uint32_t limit) { setSpinLimitOfUnit(limit); }

} // namespace pe
