// Contact solver on a thread-block cluster: the single-block solver's colour
// phases spread over kClusterRanks SMs.
//
// The single-block solver (k_solve_block) runs every colour phase of the
// velocity iterations on one SM; a phase then waits on that SM's loads of the
// prepared constants of a few hundred manifolds.  Here, in one launch:
//
//   1. ranks 1.. compute the manifolds' body flags; then rank 0 assigns
//      staging slots, colours and orders the manifolds (the single-block
//      front) while ranks 1.. prepare every manifold (by manifold index, into
//      the solver arrays);
//   2. every rank copies the prepared constants of its share of each colour
//      (solve indices start + rank, start + rank + R, ...) into its own shared
//      memory, and the velocities of its share of the staging slots (slot s
//      lives in rank s % R at s / R);
//   3. warm start and iterations colour by colour: each manifold reads and
//      writes its two bodies' velocities in the owning ranks' shared memory
//      (distributed shared memory), cluster barrier between colours;
//   4. velocities and impulses back to global memory; the ranks rebuild the
//      warm-start cache (each its share of the manifolds).
//
// Manifolds of one colour share no dynamic body and static bodies are never
// written, so spreading a colour over ranks changes no result: the arithmetic
// and the (colour, index) order are those of the single-block solver.
#include <cooperative_groups.h>

#include "pe_block.cuh"
#include "pe_kernels.cuh"
#include "pe_solve.cuh"
#include "pe_stages.h"

namespace pe {

namespace cg = cooperative_groups;

constexpr uint32_t kNoLocal = 0xFFFFFFFFu;

// Velocities of the staged bodies, spread over the cluster's shared memory.
struct ClusterVel {
    float4 *v;           // this rank's slice: slot s (s % R == rank) at 2 (s / R), 2 (s / R) + 1
    const uint2 *slot;   // [local manifold] staging slots of body A / body B
    __device__ __forceinline__ uint2 bodies(uint32_t L, uint32_t) const { return slot[L]; }
    __device__ __forceinline__ float4 *at(uint32_t s) const {
        float4 *base = cg::this_cluster().map_shared_rank(v, (int)(s % kClusterRanks));
        return base + 2 * (s / kClusterRanks);
    }
    __device__ __forceinline__ V3 lin(uint32_t s) const { return f4xyz(at(s)[0]); }
    __device__ __forceinline__ V3 ang(uint32_t s) const { return f4xyz(at(s)[1]); }
    __device__ __forceinline__ void store(uint32_t s, const V3 &l, const V3 &w) const {
        float4 *p = at(s);
        p[0] = make4(l, 0.0f);
        p[1] = make4(w, 0.0f);
    }
};

// Prepared data of this rank's manifolds (local index L) in shared memory;
// points that did not fit stay in the solver arrays.
struct LocalPrep {
    const SolveArgs &a;
    const float4 *spm, *spn;
    const uint32_t *sm, *scnt, *soff;
    float4 *spt;  // [11][pcap]: 10 prepared vectors, then the impulse
    uint32_t pcap;
    __device__ __forceinline__ float4 pm(uint32_t L) const { return spm[L]; }
    __device__ __forceinline__ float4 pn(uint32_t L) const { return spn[L]; }
    __device__ __forceinline__ uint32_t count(uint32_t L) const { return scnt[L]; }
    __device__ __forceinline__ float4 inertia(int r, uint32_t L) const {
        return __ldcg(&a.sb.pmInertia[(size_t)r * a.mcap + sm[L]]);
    }
    __device__ __forceinline__ float4 pt(int v, uint32_t p, uint32_t L) const {
        const uint32_t o = soff[L];
        return o != kNoLocal ? spt[(size_t)v * pcap + o + p] : __ldcg(&a.sb.pp[(size_t)(v * 4 + p) * a.mcap + sm[L]]);
    }
    __device__ __forceinline__ float4 imp(uint32_t p, uint32_t L) const {
        const uint32_t o = soff[L];
        return o != kNoLocal ? spt[(size_t)10 * pcap + o + p] : __ldcg(&a.sb.pimp[(size_t)p * a.mcap + sm[L]]);
    }
    __device__ __forceinline__ void setImp(uint32_t p, uint32_t L, const float4 &v) const {
        const uint32_t o = soff[L];
        if (o != kNoLocal) spt[(size_t)10 * pcap + o + p] = v;
        else a.sb.pimp[(size_t)p * a.mcap + sm[L]] = v;
    }
};

// ------------------------------------------------------------- islands ---
// Manifolds joined by a shared dynamic body form an island (static bodies are
// never written, so they join nothing; the reference's own island rule,
// sequential_impulse_solver.cpp:366-442).  Islands share no written state, and
// the graph colouring of a manifold depends only on the manifolds of its
// island (its neighbours all are), so one thread can colour a small island
// (greedy in decreasing priority: the Jones-Plassmann result), order it by
// (colour, index) and run every sweep of it on its own, with no barrier: each
// body then sees exactly the updates, in the order, that the colour-phase
// sweeps give it.
constexpr uint32_t kNoIsland = 0xFFFFFFFFu;
constexpr uint32_t kIslandUniteLimit = 1u << 16;

__device__ __forceinline__ uint32_t islandFind(const uint32_t *parent, uint32_t x) {
    uint32_t p = *(volatile const uint32_t *)&parent[x];
    for (uint32_t hops = 0; p != x && hops < kIslandUniteLimit; ++hops) {
        x = p;
        p = *(volatile const uint32_t *)&parent[x];
    }
    return x;
}

// Lock-free union (the larger root is linked under the smaller); bounded.
__device__ __forceinline__ bool islandUnite(uint32_t *parent, uint32_t a, uint32_t b) {
    for (uint32_t tries = 0; tries < kIslandUniteLimit; ++tries) {
        a = islandFind(parent, a);
        b = islandFind(parent, b);
        if (a == b) return true;
        if (a < b) {
            const uint32_t t = a;
            a = b;
            b = t;
        }
        if (atomicCAS(&parent[a], a, b) == a) return true;
    }
    return false;
}

// LocalPrep for manifolds whose points are all in shared memory (no per-load
// choice of the source).
struct LocalOnlyPrep {
    const SolveArgs &a;
    const float4 *spm, *spn;
    const uint32_t *sm, *scnt, *soff;
    float4 *spt;
    uint32_t pcap;
    __device__ __forceinline__ float4 pm(uint32_t L) const { return spm[L]; }
    __device__ __forceinline__ float4 pn(uint32_t L) const { return spn[L]; }
    __device__ __forceinline__ uint32_t count(uint32_t L) const { return scnt[L]; }
    __device__ __forceinline__ float4 inertia(int r, uint32_t L) const {
        return __ldcg(&a.sb.pmInertia[(size_t)r * a.mcap + sm[L]]);
    }
    __device__ __forceinline__ float4 pt(int v, uint32_t p, uint32_t L) const {
        return spt[(size_t)v * pcap + soff[L] + p];
    }
    __device__ __forceinline__ float4 imp(uint32_t p, uint32_t L) const { return spt[(size_t)10 * pcap + soff[L] + p]; }
    __device__ __forceinline__ void setImp(uint32_t p, uint32_t L, const float4 &v) const {
        spt[(size_t)10 * pcap + soff[L] + p] = v;
    }
};

struct IslandShared {
    uint32_t classCount[kIslandMax + 1], classBase[kIslandMax + 2], localUsed, pointUsed, bodyUsed, units;
};

struct ClusterShared {
    BlockSolveShared solve;
    uint32_t start[kMaxColors + 1];   // colour ranges of the solve order
    uint32_t lstart[kMaxColors + 1];  // colour ranges of this rank's local manifolds
    uint32_t colors, slots, slotted;
    IslandShared island;
};


// Warm-start cache rebuild after the sweeps (all ranks, after a cluster
// barrier): in manifold order every rank writes its interleaved share (as
// solveBlockCache does on one block); the sorted rebuild runs on rank 0.
__device__ void solveClusterCache(const SolveArgs &a, const CacheView &nc, uint32_t cacheCap, uint32_t *newCount,
                                  uint32_t M, uint32_t rank, unsigned char *smem, unsigned long long *s_sort,
                                  uint32_t *s_dyn, ClusterShared &cs) {
    const SolverBuffers &sb = a.sb;
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    if (!a.pairOrderCache) {
        if (rank != 0) return;
        solveBlockCache(a, nc, cacheCap, newCount, M, s_sort, s_dyn, cs.solve);
        return;
    }
    // Cache in manifold order (one manifold per body pair, pairs in body
    // order): every rank scans the point counts and writes its share.
    uint32_t *s_cnt = reinterpret_cast<uint32_t *>(smem);
    for (uint32_t i = tid; i < M; i += nt)
        s_cnt[i] = (__ldcg(&sb.dyn[i]) & kFlagValid) ? min(a.mv.pointCount[i], 4u) : 0u;
    __syncthreads();
    const uint32_t total = blockExclusiveScanArray(s_cnt, M, cs.solve.scan);
    for (uint32_t i = rank + kClusterRanks * tid; i < M; i += kClusterRanks * nt) {
        const uint32_t cnt = (i + 1 < M ? s_cnt[i + 1] : total) - s_cnt[i];
        cacheWriteManifold(a, nc, cacheCap, i, s_cnt[i], cnt);
    }
    if (rank == 0 && tid == 0) *newCount = total;
}



// One island, as its owning thread sees it: manifolds in solve order (colour,
// index), their colours, flags, points and local body indices, the island's
// bodies.
struct IslandPlan {
    uint32_t n, nbody, points, colors;
    uint32_t ks[kIslandMax], color[kIslandMax], fl[kIslandMax], cnt[kIslandMax];
    uint2 slot[kIslandMax];
    uint32_t body[2 * kIslandMax];
};

// Reads the island of root body r (n manifolds), colours it (greedy in
// decreasing priority: the colour is the first one free among the higher-
// priority neighbours at the dynamic bodies, the Jones-Plassmann round one
// more than theirs) and orders it by (colour, index).  Writes the colours and
// the colour statistics.
__device__ void planIsland(const SolveArgs &a, uint32_t r, uint32_t n, IslandPlan &P) {
    const SolverBuffers &sb = a.sb;
    uint32_t ks[kIslandMax], fl[kIslandMax];
    uint2 slot[kIslandMax];
    for (uint32_t j = 0; j < n; ++j) {
        const uint32_t m = __ldcg(&sb.islandList[(size_t)r * kIslandMax + j]);
        uint32_t i = j;
        for (; i > 0 && ks[i - 1] > m; --i) ks[i] = ks[i - 1];
        ks[i] = m;
    }
    P.nbody = 0;
    auto local = [&](uint32_t b) {
        for (uint32_t i = 0; i < P.nbody; ++i)
            if (P.body[i] == b) return i;
        P.body[P.nbody] = b;
        return P.nbody++;
    };
    for (uint32_t j = 0; j < n; ++j) {
        const uint32_t m = ks[j];
        fl[j] = __ldcg(&sb.dyn[m]);
        slot[j].x = local(a.mv.bodyA[m]);
        slot[j].y = local(a.mv.bodyB[m]);
    }
    uint32_t byPri[kIslandMax], color[kIslandMax];
    for (uint32_t j = 0; j < n; ++j) {
        const uint32_t p = colorPriority(ks[j]);
        uint32_t i = j;
        for (; i > 0 && colorPriority(ks[byPri[i - 1]]) < p; --i) byPri[i] = byPri[i - 1];
        byPri[i] = j;
    }
    uint32_t used[2 * kIslandMax], round[2 * kIslandMax];
    for (uint32_t i = 0; i < P.nbody; ++i) used[i] = round[i] = 0;
    uint32_t colors = 0, rounds = 0;
    for (uint32_t t = 0; t < n; ++t) {
        const uint32_t j = byPri[t];
        const bool dA = fl[j] & kFlagDynA, dB = fl[j] & kFlagDynB;
        const uint32_t mask = (dA ? used[slot[j].x] : 0u) | (dB ? used[slot[j].y] : 0u);
        const uint32_t c = __ffs(~mask) - 1;
        const uint32_t rd = max(dA ? round[slot[j].x] : 0u, dB ? round[slot[j].y] : 0u) + 1;
        color[j] = c;
        colors = max(colors, c + 1);
        rounds = max(rounds, rd);
        if (dA) {
            used[slot[j].x] |= 1u << c;
            round[slot[j].x] = max(round[slot[j].x], rd);
        }
        if (dB) {
            used[slot[j].y] |= 1u << c;
            round[slot[j].y] = max(round[slot[j].y], rd);
        }
        sb.color[ks[j]] = c;
    }
    atomicMax(&a.st->colors, colors);
    atomicMax(&a.st->colorRounds, rounds);
    // (colour, index) order
    uint32_t ord[kIslandMax];
    for (uint32_t j = 0; j < n; ++j) {
        uint32_t i = j;
        for (; i > 0 && color[ord[i - 1]] > color[j]; --i) ord[i] = ord[i - 1];
        ord[i] = j;
    }
    P.n = n;
    P.colors = colors;
    P.points = 0;
    for (uint32_t t = 0; t < n; ++t) {
        const uint32_t j = ord[t];
        P.ks[t] = ks[j];
        P.color[t] = color[j];
        P.fl[t] = fl[j];
        P.slot[t] = slot[j];
        P.cnt[t] = __ldcg(&sb.pcount[ks[j]]);
        P.points += P.cnt[t];
    }
}

// The island on its own thread (when it does not fit this rank's shared
// memory): prepared data from the solver arrays, velocities thread-local.
__device__ void solveIslandAlone(const SolveArgs &a, const IslandPlan &P) {
    const WorldView &w = a.w;
    float4 vel[4 * kIslandMax];
    for (uint32_t i = 0; i < P.nbody; ++i) {
        vel[2 * i] = ld4(&w.nxt.lin[P.body[i]]);
        vel[2 * i + 1] = ld4(&w.nxt.ang[P.body[i]]);
    }
    const GlobalPrep pr{a};
    const SharedVel v{vel, P.slot};
    for (uint32_t t = 0; t < P.n; ++t) warmStartOne(pr, t, P.ks[t], v);
    for (int it = 0; it < a.iterations; ++it)
        for (uint32_t t = 0; t < P.n; ++t) solveOne(pr, t, P.ks[t], v);
    for (uint32_t t = 0; t < P.n; ++t) {
        const uint32_t m = P.ks[t];
        for (uint32_t p = 0; p < P.cnt[t]; ++p) {
            float4 imp = pr.imp(p, m);
            imp.w = 0.0f;
            a.mv.impulse[4 * m + p] = imp;
        }
        if (P.fl[t] & kFlagDynA) {
            st4(&w.nxt.lin[P.body[P.slot[t].x]], vel[2 * P.slot[t].x]);
            st4(&w.nxt.ang[P.body[P.slot[t].x]], vel[2 * P.slot[t].x + 1]);
        }
        if (P.fl[t] & kFlagDynB) {
            st4(&w.nxt.lin[P.body[P.slot[t].y]], vel[2 * P.slot[t].y]);
            st4(&w.nxt.ang[P.body[P.slot[t].y]], vel[2 * P.slot[t].y + 1]);
        }
    }
}

// Island sweeps of one rank.  Islands are packed into warp-sized units by
// size (32 / n islands of n manifolds per unit, one manifold per lane); a
// warp runs a unit colour phase by colour phase (__syncwarp between phases),
// so an island's manifolds of one colour run side by side and islands of a
// unit run together.  Each manifold's prepared data and each island's body
// velocities sit in this rank's shared memory.  ownRoot: the island this
// thread owns (kNoIsland if none).
constexpr uint32_t kIslandUnits = 32;  // warp units per rank

__device__ void solveIslandsRank(const SolveArgs &a, const ClusterSolveLayout &lay, unsigned char *smem, uint32_t ownRoot,
                                 IslandShared &is, bool stamper) {
    const SolverBuffers &sb = a.sb;
    const WorldView &w = a.w;
    const uint32_t tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
    float4 *spm = reinterpret_cast<float4 *>(smem + lay.offPm);
    float4 *spn = reinterpret_cast<float4 *>(smem + lay.offPn);
    float4 *spt = reinterpret_cast<float4 *>(smem + lay.offPt);
    uint2 *sslot = reinterpret_cast<uint2 *>(smem + lay.offSlot);
    uint32_t *sm = reinterpret_cast<uint32_t *>(smem + lay.offM);
    uint32_t *scnt = reinterpret_cast<uint32_t *>(smem + lay.offCnt);
    uint32_t *soff = reinterpret_cast<uint32_t *>(smem + lay.offOff);
    float4 *sv = reinterpret_cast<float4 *>(smem + lay.offVel);                      // [2 * islandBodies]
    uint32_t *laneL = reinterpret_cast<uint32_t *>(smem + lay.offVel + (size_t)lay.islandBodies * 32);
    uint32_t *unitC = laneL + kIslandUnits * 32;
    uint32_t *scol = unitC + kIslandUnits;                                             // [localCap]
    if (tid <= kIslandMax) is.classCount[tid] = 0;
    if (tid == 0) is.localUsed = is.pointUsed = is.bodyUsed = 0;
    for (uint32_t i = tid; i < kIslandUnits * 32; i += nt) laneL[i] = kNoLocal;
    for (uint32_t i = tid; i < kIslandUnits; i += nt) unitC[i] = 0;
    __syncthreads();
    IslandPlan P;
    uint32_t idx = 0;
    if (ownRoot != kNoIsland) {
        planIsland(a, ownRoot, __ldcg(&reinterpret_cast<uint32_t *>(sb.bodyUsed)[w.nb + ownRoot]), P);
        idx = atomicAdd(&is.classCount[P.n], 1u);
    }
    __syncthreads();
    if (tid == 0) {
        uint32_t base = 0;
        for (uint32_t c = 1; c <= kIslandMax; ++c) {
            is.classBase[c] = base;
            const uint32_t per = 32 / c;
            base += (is.classCount[c] + per - 1) / per;
        }
        is.units = base;
    }
    __syncthreads();
    bool packed = false;
    uint32_t L0 = 0, B0 = 0;
    if (ownRoot != kNoIsland) {
        const uint32_t per = 32 / P.n;
        const uint32_t u = is.classBase[P.n] + idx / per, lane0 = (idx % per) * P.n;
        if (u < kIslandUnits) {
            L0 = atomicAdd(&is.localUsed, P.n);
            const uint32_t P0 = atomicAdd(&is.pointUsed, P.points);
            B0 = atomicAdd(&is.bodyUsed, P.nbody);
            packed = L0 + P.n <= lay.localCap && P0 + P.points <= lay.pointCap && B0 + P.nbody <= lay.islandBodies;
            if (packed) {
                uint32_t o = P0;
                for (uint32_t t = 0; t < P.n; ++t) {
                    const uint32_t m = P.ks[t], L = L0 + t;
                    sm[L] = m;
                    sslot[L] = make_uint2(B0 + P.slot[t].x, B0 + P.slot[t].y);
                    spm[L] = __ldcg(&sb.pm[m]);
                    spn[L] = __ldcg(&sb.pn[m]);
                    scnt[L] = P.cnt[t];
                    soff[L] = o;
                    scol[L] = P.color[t];
                    for (uint32_t p = 0; p < P.cnt[t]; ++p) {
#pragma unroll
                        for (int v = 0; v < kPreparedVec4; ++v)
                            spt[(size_t)v * lay.pointCap + o + p] = __ldcg(&sb.pp[(size_t)(v * 4 + p) * a.mcap + m]);
                        spt[(size_t)10 * lay.pointCap + o + p] = __ldcg(&sb.pimp[(size_t)p * a.mcap + m]);
                    }
                    o += P.cnt[t];
                    laneL[u * 32 + lane0 + t] = L;
                }
                for (uint32_t i = 0; i < P.nbody; ++i) {
                    sv[2 * (B0 + i)] = ld4(&w.nxt.lin[P.body[i]]);
                    sv[2 * (B0 + i) + 1] = ld4(&w.nxt.ang[P.body[i]]);
                }
                atomicMax(&unitC[u], P.colors);
            }
        }
        if (!packed) solveIslandAlone(a, P);
    }
    __syncthreads();
    if (stamper) a.st->solverStamp[4] = globalNs();
    // warp units: pass by pass (pass 0: warm start), colour by colour
    const LocalOnlyPrep pr{a, spm, spn, sm, scnt, soff, spt, lay.pointCap};
    const SharedVel v{sv, sslot};
    for (uint32_t u = warp; u < min(is.units, kIslandUnits); u += nt >> 5) {
        const uint32_t L = laneL[u * 32 + lane], C = unitC[u];
        const uint32_t c = L != kNoLocal ? scol[L] : kNoLocal;
        for (int pass = 0; pass <= a.iterations; ++pass)
            for (uint32_t cc = 0; cc < C; ++cc) {
                if (c == cc) {
                    if (pass == 0) warmStartOne(pr, L, L, v);
                    else solveOne(pr, L, L, v);
                }
                __syncwarp();
            }
    }
    __syncthreads();
    if (stamper) a.st->solverStamp[5] = globalNs();
    if (packed) {
        for (uint32_t t = 0; t < P.n; ++t) {
            const uint32_t m = P.ks[t], L = L0 + t;
            for (uint32_t p = 0; p < P.cnt[t]; ++p) {
                float4 imp = pr.imp(p, L);
                imp.w = 0.0f;
                a.mv.impulse[4 * m + p] = imp;
            }
            if (P.fl[t] & kFlagDynA) {
                const uint32_t i = B0 + P.slot[t].x;
                st4(&w.nxt.lin[P.body[P.slot[t].x]], sv[2 * i]);
                st4(&w.nxt.ang[P.body[P.slot[t].x]], sv[2 * i + 1]);
            }
            if (P.fl[t] & kFlagDynB) {
                const uint32_t i = B0 + P.slot[t].y;
                st4(&w.nxt.lin[P.body[P.slot[t].y]], sv[2 * i]);
                st4(&w.nxt.ang[P.body[P.slot[t].y]], sv[2 * i + 1]);
            }
        }
    }
}

__global__ void __cluster_dims__(kClusterRanks, 1, 1) __launch_bounds__(kBlockSolveThreads, 1)
k_solve_cluster(SolveArgs a, CacheView nc, uint32_t cacheCap, uint32_t *newCount, ClusterSolveLayout lay) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ ClusterShared cs;
    cg::cluster_group cluster = cg::this_cluster();
    const uint32_t rank = cluster.block_rank();
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    const SolverBuffers &sb = a.sb;
    const WorldView &w = a.w;
    const uint32_t M = min(*a.count, a.mcap);
    if (M > lay.blockM) {  // every rank sees the same count
        if (rank == 0 && tid == 0) atomicOr(&a.st->err, kErrSmallPath);
        return;
    }
    const bool stamper = rank == 0 && tid == 0;
    auto stamp = [&](int k) {
        if (stamper) a.st->solverStamp[k] = globalNs();
    };
    stamp(0);

    // ---- 0. all ranks: manifold flags, island sets, prepare ----
    // (manifolds spread over all SMs: their scattered loads are what costs time)
    const uint32_t g = tid * kClusterRanks + rank, G = kClusterRanks * nt;  // consecutive manifolds: other SMs
    uint32_t *par = reinterpret_cast<uint32_t *>(sb.bodyUsed);  // island parent of a body
    uint32_t *icnt = par + w.nb;                                 // manifolds of an island, at its root
    if (g == 0) sb.counters[2] = 0;                              // island path refused
    for (uint32_t m = g; m < M; m += G) {
        const uint32_t fl = manifoldFlags(a, m);
        sb.dyn[m] = fl;
        if (fl & kFlagValid) {
            const uint32_t ba = a.mv.bodyA[m], bb = a.mv.bodyB[m];
            if (fl & kFlagDynA) {
                par[ba] = ba;
                icnt[ba] = 0;
            }
            if (fl & kFlagDynB) {
                par[bb] = bb;
                icnt[bb] = 0;
            }
        }
    }
    unsigned long long *s_sort = reinterpret_cast<unsigned long long *>(smem);
    uint32_t *s_dyn = reinterpret_cast<uint32_t *>(smem + (size_t)lay.blockM * 8);
    {
        // old cache keys in this rank's shared memory when they fit
        const uint32_t cacheN = *a.oldCount;
        const bool keysInShared = (size_t)cacheN * 8 <= lay.smemBytes;
        if (keysInShared)
            for (uint32_t i = tid; i < cacheN; i += nt) s_sort[i] = a.oldCache.key[i];
        __syncthreads();
        prepareRange(a, g, G, M, keysInShared ? s_sort : nullptr);
    }
    __threadfence();
    cluster.sync();
    stamp(1);
    // ---- 1. islands: union of the two dynamic bodies of every solved manifold ----
    for (uint32_t m = g; m < M; m += G) {
        const uint32_t fl = __ldcg(&sb.dyn[m]);
        if ((fl & (kFlagValid | kFlagDynA | kFlagDynB)) == (kFlagValid | kFlagDynA | kFlagDynB))
            if (!islandUnite(par, a.mv.bodyA[m], a.mv.bodyB[m])) atomicOr(&sb.counters[2], 1u);
    }
    __threadfence();
    cluster.sync();
    stamp(2);
    // ---- 2. each solved manifold joins its island's list; the first to join
    // owns the island (M <= blockM <= threads of the cluster: one manifold per
    // thread) ----
    uint32_t ownRoot = kNoIsland;
    for (uint32_t m = g; m < M; m += G) {
        const uint32_t fl = __ldcg(&sb.dyn[m]);
        if (!(fl & kFlagValid)) {
            // an unsolved manifold that still shapes the colouring: colour-phase path
            if (fl & (kFlagDynA | kFlagDynB)) atomicOr(&sb.counters[2], 1u);
            continue;
        }
        if (!(fl & (kFlagDynA | kFlagDynB))) {
            atomicOr(&sb.counters[2], 1u);  // solved manifold without a dynamic body
            continue;
        }
        const uint32_t r = islandFind(par, (fl & kFlagDynA) ? a.mv.bodyA[m] : a.mv.bodyB[m]);
        const uint32_t pos = atomicAdd(&icnt[r], 1u);
        if (pos < kIslandMax) sb.islandList[(size_t)r * kIslandMax + pos] = m;
        else atomicOr(&sb.counters[2], 1u);
        if (pos == 0) ownRoot = r;
    }
    __threadfence();
    cluster.sync();
    stamp(3);
    // The island path needs the cache in manifold order (one manifold per body
    // pair): a cache sorted over the solve order needs the order, which only
    // the colour-phase path materialises.
    if (__ldcg(&sb.counters[2]) == 0 && G >= M && a.pairOrderCache) {
        // ---- island path ----
        if (g == 0) atomicMax(&a.st->colorRounds, 1u);  // one round when nothing is coloured
        solveIslandsRank(a, lay, smem, ownRoot, cs.island, stamper);
        __threadfence();
        cluster.sync();
        stamp(6);
        solveClusterCache(a, nc, cacheCap, newCount, M, rank, smem, s_sort, s_dyn, cs);
        stamp(7);
        return;
    }

    // ---- colour-phase path: rank 0 assigns slots, colours and orders ----
    if (rank == 0) {
        VelStage vs;
        vs.slot = reinterpret_cast<uint2 *>(smem + (size_t)lay.blockM * 12);
        vs.v = reinterpret_cast<float4 *>(smem + (size_t)lay.blockM * 20);
        vs.slotBody = reinterpret_cast<uint32_t *>(smem + (size_t)lay.blockM * 20 + (size_t)lay.stageSlots * 32);
        vs.cap = lay.stageSlots;
        const bool slotted = solveBlockFront(a, M, 0, lay.blockM, s_sort, s_dyn, cs.solve, &vs, sb.dyn);
        if (slotted) {
            for (uint32_t k = tid; k < M; k += nt) sb.stageSlot[k] = vs.slot[k];
            for (uint32_t sl = tid; sl < cs.solve.slots; sl += nt) sb.stageBody[sl] = vs.slotBody[sl];
        }
        if (tid == 0) {
            sb.counters[0] = slotted ? cs.solve.slots : 0u;
            sb.counters[1] = slotted ? 1u : 0u;
        }
    }
    __threadfence();
    cluster.sync();
    stamp(4);
    if (__ldcg(&a.st->colors) > (uint32_t)kMaxColors) {
        // More colours than the cluster's shared colour ranges hold (a body
        // touching more than ~64 others): the step is re-run on the
        // multi-kernel path.  Every rank reads the same count.
        if (rank == 0 && tid == 0) atomicOr(&a.st->err, kErrSmallPath);
        return;
    }

    // ---- 2. this rank's share of every colour and of the staging slots ----
    if (tid == 0) {
        cs.slotted = __ldcg(&sb.counters[1]);
        cs.slots = __ldcg(&sb.counters[0]);
        const uint32_t C = min(__ldcg(&a.st->colors), (uint32_t)kMaxColors);
        cs.colors = C;
        uint32_t acc = 0, lacc = 0;
        for (uint32_t c = 0; c < C; ++c) {
            const uint32_t cnt = __ldcg(&sb.colorCount[c]);
            cs.start[c] = acc;
            cs.lstart[c] = lacc;
            acc += cnt;
            lacc += cnt > rank ? (cnt - rank + kClusterRanks - 1) / kClusterRanks : 0u;
        }
        cs.start[C] = acc;
        cs.lstart[C] = lacc;
    }
    __syncthreads();
    if (!cs.slotted) {
        // Too many bodies to stage: rank 0 runs the single-block sweeps on the
        // world's velocity arrays (the order is in its s_dyn).
        if (rank != 0) return;
        solveBlockSweeps(a, M, 0, cs.solve.colors, false, s_dyn, cs.solve, nullptr);
        solveBlockCache(a, nc, cacheCap, newCount, M, s_sort, s_dyn, cs.solve);
        return;
    }
    float4 *sv = reinterpret_cast<float4 *>(smem + lay.offVel);
    float4 *spm = reinterpret_cast<float4 *>(smem + lay.offPm);
    float4 *spn = reinterpret_cast<float4 *>(smem + lay.offPn);
    float4 *spt = reinterpret_cast<float4 *>(smem + lay.offPt);
    uint2 *sslot = reinterpret_cast<uint2 *>(smem + lay.offSlot);
    uint32_t *sm = reinterpret_cast<uint32_t *>(smem + lay.offM);
    uint32_t *scnt = reinterpret_cast<uint32_t *>(smem + lay.offCnt);
    uint32_t *soff = reinterpret_cast<uint32_t *>(smem + lay.offOff);
    const uint32_t C = cs.colors, Lr = cs.lstart[C], S = cs.slots;
    if (Lr > lay.localCap) {  // cannot happen: localCap covers blockM / R + one per colour
        if (tid == 0) atomicOr(&a.st->err, kErrSmallPath);
    }
    const uint32_t L1 = min(Lr, lay.localCap);
    for (uint32_t L = tid; L < L1; L += nt) {
        uint32_t c = 0;
        while (c + 1 < C && cs.lstart[c + 1] <= L) ++c;
        const uint32_t k = cs.start[c] + rank + kClusterRanks * (L - cs.lstart[c]);
        const uint32_t m = __ldcg(&sb.order[k]);
        sm[L] = m;
        sslot[L] = __ldcg(&sb.stageSlot[k]);
        spm[L] = __ldcg(&sb.pm[m]);
        spn[L] = __ldcg(&sb.pn[m]);
        scnt[L] = __ldcg(&sb.pcount[m]);
        soff[L] = scnt[L];
    }
    for (uint32_t i = tid; rank + kClusterRanks * i < S; i += nt) {
        const uint32_t b = __ldcg(&sb.stageBody[rank + kClusterRanks * i]);
        sv[2 * i] = ld4(&w.nxt.lin[b]);
        sv[2 * i + 1] = ld4(&w.nxt.ang[b]);
    }
    __syncthreads();
    // point offsets; points past the local capacity stay in global memory
    blockExclusiveScanArray(soff, L1, cs.solve.scan);
    for (uint32_t L = tid; L < L1; L += nt) {
        const uint32_t o = soff[L], n = scnt[L], m = sm[L];
        if (o + n > lay.pointCap) {
            soff[L] = kNoLocal;
            continue;
        }
        for (uint32_t p = 0; p < n; ++p) {
#pragma unroll
            for (int v = 0; v < kPreparedVec4; ++v)
                spt[(size_t)v * lay.pointCap + o + p] = __ldcg(&sb.pp[(size_t)(v * 4 + p) * a.mcap + m]);
            spt[(size_t)10 * lay.pointCap + o + p] = __ldcg(&sb.pimp[(size_t)p * a.mcap + m]);
        }
    }
    cluster.sync();  // every slice loaded before any rank reads another's

    // ---- 3. warm start and iterations, colour by colour ----
    const LocalPrep pr{a, spm, spn, sm, scnt, soff, spt, lay.pointCap};
    const ClusterVel cv{sv, sslot};
    for (uint32_t c = 0; c < C; ++c) {
        for (uint32_t L = cs.lstart[c] + tid; L < cs.lstart[c + 1]; L += nt) warmStartOne(pr, L, L, cv);
        cluster.sync();
    }
    for (int it = 0; it < a.iterations; ++it)
        for (uint32_t c = 0; c < C; ++c) {
            for (uint32_t L = cs.lstart[c] + tid; L < cs.lstart[c + 1]; L += nt) solveOne(pr, L, L, cv);
            cluster.sync();
        }
    stamp(5);

    // ---- 4. velocities and impulses back; the warm-start cache ----
    for (uint32_t i = tid; rank + kClusterRanks * i < S; i += nt) {
        const uint32_t b = __ldcg(&sb.stageBody[rank + kClusterRanks * i]);
        st4(&w.nxt.lin[b], sv[2 * i]);
        st4(&w.nxt.ang[b], sv[2 * i + 1]);
    }
    for (uint32_t L = tid; L < L1; L += nt) {
        const uint32_t m = sm[L], n = scnt[L];
        for (uint32_t p = 0; p < n; ++p) {
            float4 imp = pr.imp(p, L);
            imp.w = 0.0f;
            a.mv.impulse[4 * m + p] = imp;
        }
    }
    __threadfence();
    cluster.sync();
    stamp(6);
    solveClusterCache(a, nc, cacheCap, newCount, M, rank, smem, s_sort, s_dyn, cs);
    stamp(7);
}

// Layout of one rank's dynamic shared memory (kClusterSmemMax bytes): the
// single-block front (blockM * 20 + stageSlots * 36 bytes, rank 0) and,
// afterwards, in the same bytes, the velocity slice, the local manifolds and
// as many prepared points (176 bytes each) as fit.
ClusterSolveLayout clusterSolveLayout(uint32_t blockM, uint32_t stageSlots) {
    ClusterSolveLayout l{};
    l.blockM = blockM;
    l.stageSlots = stageSlots;
    const size_t front = (size_t)blockM * 20 + (size_t)stageSlots * 36;
    const uint32_t velSlots = (stageSlots + kClusterRanks - 1) / kClusterRanks;
    l.localCap = (blockM + kClusterRanks - 1) / kClusterRanks + kMaxColors;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off += (bytes + 15) & ~(size_t)15;
        return (uint32_t)o;
    };
    // the velocity area: this rank's slice of the staged velocities (colour-
    // phase path) or the islands' body velocities, unit lane maps and colours
    // (island path)
    l.islandBodies = 2 * l.localCap;
    const size_t islandArea = (size_t)l.islandBodies * 32 + (kIslandUnits * 32 + kIslandUnits) * 4 + (size_t)l.localCap * 4;
    l.offVel = take(std::max<size_t>((size_t)velSlots * 32, islandArea));
    l.offPm = take((size_t)l.localCap * 16);
    l.offPn = take((size_t)l.localCap * 16);
    l.offSlot = take((size_t)l.localCap * 8);
    l.offM = take((size_t)l.localCap * 4);
    l.offCnt = take((size_t)l.localCap * 4);
    l.offOff = take((size_t)l.localCap * 4);
    l.offPt = (uint32_t)off;
    // one rank per SM in any case: take the SM's shared memory
    l.smemBytes = kClusterSmemMax;
    l.pointCap = off < kClusterSmemMax ? (uint32_t)((kClusterSmemMax - off) / 176) : 0u;
    if (front > kClusterSmemMax) l.smemBytes = 0;  // does not fit: no cluster launch
    return l;
}

bool launchSolverCluster(const SolveArgs &a, const CacheView &newCache, uint32_t *newCacheCount, uint32_t cacheCap,
                         uint32_t blockM, uint32_t stageSlots, cudaStream_t s) {
    static int usable = -1;
    const ClusterSolveLayout lay = clusterSolveLayout(blockM, stageSlots);
    if (usable < 0) {
        usable = 0;
        if (cudaFuncSetAttribute(k_solve_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kClusterSmemMax) ==
            cudaSuccess) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(kClusterRanks);
            cfg.blockDim = dim3(kBlockSolveThreads);
            cfg.dynamicSmemBytes = kClusterSmemMax;
            int clusters = 0;
            if (cudaOccupancyMaxActiveClusters(&clusters, k_solve_cluster, &cfg) == cudaSuccess && clusters > 0)
                usable = 1;
        }
        cudaGetLastError();  // a refused query leaves no sticky error
    }
    if (!usable || lay.smemBytes == 0) return false;
    k_solve_cluster<<<kClusterRanks, kBlockSolveThreads, lay.smemBytes, s>>>(a, newCache, cacheCap, newCacheCount, lay);
    PE_LAUNCHED();
    return true;
}

} // namespace pe
