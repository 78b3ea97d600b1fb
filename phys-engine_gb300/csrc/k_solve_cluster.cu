// Contact solver on a thread-block cluster of kClusterRanks SMs, for steps of
// at most kBlockMaxManifolds manifolds.  In one launch:
//
//   0. all ranks prepare every manifold (by manifold index, into the solver
//      arrays), compute the manifolds' body flags and unite the two dynamic
//      bodies of every solved manifold (union-find over bodies);
//   1. each solved manifold appends a record to its island's list (the root
//      body's); cluster barrier;
//   2. island path (every island at most kIslandMax manifolds): the owner of
//      each island colours and orders it and stages its prepared data and
//      body velocities in its rank's shared memory; warps run packed islands
//      colour phase by colour phase and write their results and warm-start
//      cache entries themselves (no barrier beyond the warp);
//   3. colour-phase path otherwise: rank 0 assigns staging slots, colours and
//      orders every manifold (the single-block front); every rank copies the
//      prepared constants of its share of each colour (solve indices start +
//      rank, start + rank + R, ...) and the velocities of its share of the
//      staging slots (slot s lives in rank s % R at s / R) into its shared
//      memory; warm start and iterations run colour by colour, each manifold
//      reading and writing its two bodies' velocities in the owning ranks'
//      shared memory (distributed shared memory), a cluster barrier between
//      colours; then velocities, impulses and the warm-start cache.
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

// Union-find over bodies with each link stored as parent XOR body: a root's
// link is 0, so the zero-filled array holds every body as its own island and
// the first unions need no initialisation pass (and no barrier after one).
// The solver sets every link it wrote back to 0 before it ends.  A link always
// points to a smaller body index, so there are no cycles.
//
// Union: link the larger of the two under the smaller by one compare-and-swap
// when it is a root (the common case: one memory round trip); otherwise move
// to its parent and try again.  Each try lowers the larger index, so it ends.
__device__ __forceinline__ bool islandUnite(uint32_t *link, uint32_t a, uint32_t b) {
    for (uint32_t tries = 0; tries < kIslandUniteLimit; ++tries) {
        if (a == b) return true;
        if (a < b) {
            const uint32_t t = a;
            a = b;
            b = t;
        }
        const uint32_t old = atomicCAS(&link[a], 0u, a ^ b);
        if (old == 0u) return true;
        a ^= old;  // a's parent
    }
    return false;
}

// Root of x once every union is done, halving the path on the way (each node
// passed is pointed at its grandparent, still an ancestor, so concurrent finds
// shorten chains for one another).
__device__ __forceinline__ uint32_t islandFind(uint32_t *link, uint32_t x) {
    for (uint32_t hops = 0; hops < kIslandUniteLimit; ++hops) {
        const uint32_t p = *(volatile const uint32_t *)&link[x] ^ x;
        if (p == x) return x;
        const uint32_t gp = *(volatile const uint32_t *)&link[p] ^ p;
        if (gp == p) return p;
        link[x] = gp ^ x;
        x = gp;
    }
    return x;
}

// Island record word 0: manifold index, its flags and its solved point count.
constexpr uint32_t kRecManifoldMask = (1u << 13) - 1u;
static_assert(kBlockMaxManifolds <= kRecManifoldMask + 1u, "island record: manifold index field too narrow");
static_assert(kBlockMaxManifolds <= kClusterRanks * kBlockSolveThreads, "one manifold per cluster thread");
__device__ __forceinline__ uint32_t islandRecWord(uint32_t m, uint32_t fl, uint32_t points) {
    return m | fl << 13 | points << 16;
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

// LocalOnlyPrep with one manifold's inverse inertia rows in registers (the
// warm start's only reads from global memory).
struct InertiaInRegs {
    const LocalOnlyPrep &p;
    float4 r[6];
    __device__ __forceinline__ float4 pm(uint32_t L) const { return p.pm(L); }
    __device__ __forceinline__ float4 pn(uint32_t L) const { return p.pn(L); }
    __device__ __forceinline__ uint32_t count(uint32_t L) const { return p.count(L); }
    __device__ __forceinline__ float4 inertia(int j, uint32_t) const { return r[j]; }
    __device__ __forceinline__ float4 pt(int v, uint32_t q, uint32_t L) const { return p.pt(v, q, L); }
    __device__ __forceinline__ float4 imp(uint32_t q, uint32_t L) const { return p.imp(q, L); }
    __device__ __forceinline__ void setImp(uint32_t q, uint32_t L, const float4 &v) const { p.setImp(q, L, v); }
};

struct IslandShared {
    uint32_t classCount[kIslandMax + 1], classBase[kIslandMax + 2], localUsed, pointUsed, bodyUsed, units, plans;
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



// One island, as its owning thread plans it: manifolds in solve order
// (colour, index) with, per manifold, its colour, point count and local body
// indices (meta: colour | points << 8 | local A << 16 | local B << 24), the
// island's bodies and which of them are dynamic (written back); and the
// planner's working arrays in manifold order.  A plan lives in shared memory
// (the prepared-point area, free until the staging), so that its dependent
// reads and writes cost no trip to memory.
struct IslandPlan {
    uint32_t n, nbody, points, colors, dynMask;
    uint32_t ks[kIslandMax], meta[kIslandMax];
    uint32_t body[2 * kIslandMax];
    uint32_t wm[kIslandMax], wmeta[kIslandMax];  // manifold order: index; flags | points << 3 | colour << 8 | slots
    uint32_t ur[2 * kIslandMax];                 // per body: colours used (bits 0-15) | round << 16
};
__device__ __forceinline__ uint32_t planColor(uint32_t meta) { return meta & 0xFFu; }
__device__ __forceinline__ uint32_t planPoints(uint32_t meta) { return (meta >> 8) & 0xFFu; }
__device__ __forceinline__ uint2 planSlots(uint32_t meta) { return make_uint2((meta >> 16) & 0xFFu, meta >> 24); }

// Reads the n records of one island, colours it (greedy in decreasing
// priority: the colour is the first one free among the higher-priority
// neighbours at the dynamic bodies, the Jones-Plassmann round one more than
// theirs) and orders it by (colour, index).  Writes the colours and the colour
// statistics.  Orders are built by counting (priorities are distinct: the
// priority hash is a bijection of the manifold index).
__device__ void planIsland(const SolveArgs &a, const uint4 *rec, uint32_t n, IslandPlan &P) {
    const SolverBuffers &sb = a.sb;
    if (n == 1) {
        // one manifold: colour 0, one round, bodies A and B
        const uint4 r0 = __ldcg(&rec[0]);
        const uint32_t m = r0.x & kRecManifoldMask, fl = (r0.x >> 13) & 7u, pts = (r0.x >> 16) & 7u;
        P.n = 1;
        P.nbody = 2;
        P.body[0] = r0.y;
        P.body[1] = r0.z;
        P.dynMask = ((fl & kFlagDynA) ? 1u : 0u) | ((fl & kFlagDynB) ? 2u : 0u);
        P.ks[0] = m;
        P.meta[0] = pts << 8 | 1u << 24;
        P.points = pts;
        P.colors = 1;
        sb.color[m] = 0;
        atomicMax(&a.st->colors, 1u);
        return;
    }
    uint4 r[kIslandMax];
#pragma unroll
    for (uint32_t j = 0; j < kIslandMax; ++j)
        if (j < n) r[j] = __ldcg(&rec[j]);  // every record requested at once
    // manifold order: position of record j = records with a smaller index
#pragma unroll
    for (uint32_t j = 0; j < kIslandMax; ++j)
        if (j < n) P.wm[j] = r[j].x;
    P.nbody = 0;
    P.dynMask = 0;
    auto local = [&](uint32_t b) {
        for (uint32_t i = 0; i < P.nbody; ++i)
            if (P.body[i] == b) return i;
        P.body[P.nbody] = b;
        P.ur[P.nbody] = 0;
        return P.nbody++;
    };
    uint32_t sortedA[kIslandMax], sortedB[kIslandMax];
#pragma unroll
    for (uint32_t j = 0; j < kIslandMax; ++j) {
        if (j >= n) continue;
        uint32_t pos = 0;
        for (uint32_t i = 0; i < n; ++i) pos += (P.wm[i] & kRecManifoldMask) < (r[j].x & kRecManifoldMask);
        P.wmeta[pos] = j;  // record of position pos
        sortedA[j] = r[j].y;
        sortedB[j] = r[j].z;
    }
    for (uint32_t t = 0; t < n; ++t) {
        const uint32_t j = P.wmeta[t];
        uint32_t w0 = 0, ba = 0, bb = 0;
#pragma unroll
        for (uint32_t i = 0; i < kIslandMax; ++i)
            if (i == j) {
                w0 = r[i].x;
                ba = sortedA[i];
                bb = sortedB[i];
            }
        const uint32_t fl = (w0 >> 13) & 7u, pts = (w0 >> 16) & 7u;
        const uint32_t sa = local(ba), sbb = local(bb);
        if (fl & kFlagDynA) P.dynMask |= 1u << sa;
        if (fl & kFlagDynB) P.dynMask |= 1u << sbb;
        P.wmeta[t] = fl | pts << 3 | sa << 16 | sbb << 24;
        P.ks[t] = w0 & kRecManifoldMask;  // manifold order for now
    }
    for (uint32_t t = 0; t < n; ++t) P.wm[t] = P.ks[t];
    // priority order (meta holds it until the solve order is written)
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t pi = colorPriority(P.wm[i]);
        uint32_t rank = 0;
        for (uint32_t k = 0; k < n; ++k) rank += colorPriority(P.wm[k]) > pi;
        P.meta[rank] = i;
    }
    // colouring in decreasing priority
    uint32_t colors = 0, rounds = 0;
    for (uint32_t t = 0; t < n; ++t) {
        const uint32_t j = P.meta[t];
        const uint32_t wm = P.wmeta[j];
        const uint32_t fl = wm & 7u, sa = (wm >> 16) & 0xFFu, sbb = wm >> 24;
        const bool dA = fl & kFlagDynA, dB = fl & kFlagDynB;
        const uint32_t ua = dA ? P.ur[sa] : 0u, ub = dB ? P.ur[sbb] : 0u;
        const uint32_t mask = (ua | ub) & 0xFFFFu;
        const uint32_t c = __ffs(~mask) - 1;
        const uint32_t rd = max(ua >> 16, ub >> 16) + 1;
        P.wmeta[j] = wm | c << 8;
        colors = max(colors, c + 1);
        rounds = max(rounds, rd);
        if (dA) P.ur[sa] = ((P.ur[sa] | 1u << c) & 0xFFFFu) | max(P.ur[sa] >> 16, rd) << 16;
        if (dB) P.ur[sbb] = ((P.ur[sbb] | 1u << c) & 0xFFFFu) | max(P.ur[sbb] >> 16, rd) << 16;
        sb.color[P.wm[j]] = c;
    }
    atomicMax(&a.st->colors, colors);
    atomicMax(&a.st->colorRounds, rounds);
    // (colour, index) order: position = smaller colours + equal colours earlier
    P.n = n;
    P.colors = colors;
    P.points = 0;
    for (uint32_t j = 0; j < n; ++j) {
        const uint32_t wj = P.wmeta[j], cj = (wj >> 8) & 0xFFu;
        uint32_t pos = 0;
        for (uint32_t i = 0; i < n; ++i) {
            const uint32_t ci = (P.wmeta[i] >> 8) & 0xFFu;
            pos += ci < cj || (ci == cj && i < j);
        }
        const uint32_t pts = (wj >> 3) & 7u;
        P.ks[pos] = P.wm[j];
        P.meta[pos] = cj | pts << 8 | (wj & 0xFFFF0000u);
        P.points += pts;
    }
}

// One solved manifold's impulses into the manifold arrays and its points into
// the warm-start cache in manifold order at base (cacheWriteManifold, with the
// impulses at hand).  L: the manifold's index for pr.
template <class Prep>
__device__ __forceinline__ void writeManifoldResult(const SolveArgs &a, const CacheView &nc, uint32_t cacheCap,
                                                    const Prep &pr, uint32_t L, uint32_t m, uint32_t ba,
                                                    uint32_t bb, uint32_t npts, uint32_t base) {
    const unsigned long long key = ((unsigned long long)ba << 32) | bb;
    const unsigned long long gens = ((unsigned long long)a.mv.genA[m] << 32) | a.mv.genB[m];
    for (uint32_t p = 0; p < npts; ++p) {
        float4 imp = pr.imp(p, L);
        imp.w = 0.0f;
        a.mv.impulse[4 * m + p] = imp;
        const uint32_t e = base + p;
        if (e >= cacheCap) continue;
        const float4 aa = a.mv.anchorA[4 * m + p], ab = a.mv.anchorB[4 * m + p];
        nc.key[e] = key;
        nc.gens[e] = gens;
        nc.anchorA[e] = make_float4(aa.x, aa.y, aa.z, imp.x);
        nc.anchorB[e] = make_float4(ab.x, ab.y, ab.z, imp.y);
        nc.tangent2[e] = imp.z;
    }
}

// The island on its own thread (when it does not fit this rank's shared
// memory): prepared data from the solver arrays, velocities thread-local;
// then its results and cache entries.  P: a copy in the owner's local memory.
__device__ void solveIslandAlone(const SolveArgs &a, const CacheView &nc, uint32_t cacheCap, const uint32_t *scoff,
                                 const IslandPlan &P) {
    const WorldView &w = a.w;
    float4 vel[4 * kIslandMax];
    uint2 slot[kIslandMax];
    for (uint32_t t = 0; t < P.n; ++t) slot[t] = planSlots(P.meta[t]);
    for (uint32_t i = 0; i < P.nbody; ++i) {
        vel[2 * i] = ld4(&w.nxt.lin[P.body[i]]);
        vel[2 * i + 1] = ld4(&w.nxt.ang[P.body[i]]);
    }
    const GlobalPrep pr{a};
    const SharedVel v{vel, slot};
    for (uint32_t t = 0; t < P.n; ++t) warmStartOne(pr, t, P.ks[t], v);
    for (int it = 0; it < a.iterations; ++it)
        for (uint32_t t = 0; t < P.n; ++t) solveOne(pr, t, P.ks[t], v);
    for (uint32_t t = 0; t < P.n; ++t) {
        const uint32_t m = P.ks[t];
        writeManifoldResult(a, nc, cacheCap, pr, m, m, P.body[slot[t].x], P.body[slot[t].y], planPoints(P.meta[t]),
                            scoff[m]);
    }
    for (uint32_t i = 0; i < P.nbody; ++i)
        if (P.dynMask >> i & 1u) {
            st4(&w.nxt.lin[P.body[i]], vel[2 * i]);
            st4(&w.nxt.ang[P.body[i]], vel[2 * i + 1]);
        }
}

// Island sweeps of one rank.  Islands are packed into warp-sized units by
// size (32 / n islands of n manifolds per unit, one manifold per lane); a
// warp runs a unit colour phase by colour phase (__syncwarp between phases),
// so an island's manifolds of one colour run side by side and islands of a
// unit run together.  Each manifold's prepared data and each island's body
// velocities sit in this rank's shared memory: the owners lay out their
// islands and every thread of the rank then loads a share of the data (one
// memory round trip for the rank, not one per point of an island).  After the
// last pass the lanes write their manifolds' impulses and cache entries and
// their share of the island's bodies, with no barrier beyond the warp.
// ownRoot / ownN: the island this thread owns and its manifold count
// (kNoIsland if none).
constexpr uint32_t kIslandUnits = 32;  // warp units per rank
constexpr uint32_t kBodyNotDynamic = 0x80000000u;
constexpr uint32_t kNoBody = 0xFFFFFFFFu;

__device__ void solveIslandsRank(const SolveArgs &a, const CacheView &nc, uint32_t cacheCap, uint32_t *newCount,
                                 uint32_t M, uint32_t rank, const ClusterSolveLayout &lay, unsigned char *smem,
                                 uint32_t ownRoot, uint32_t ownN, ClusterShared &cs, bool stamper) {
    const SolverBuffers &sb = a.sb;
    const WorldView &w = a.w;
    IslandShared &is = cs.island;
    const uint32_t tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
    float4 *spm = reinterpret_cast<float4 *>(smem + lay.offPm);
    float4 *spn = reinterpret_cast<float4 *>(smem + lay.offPn);
    float4 *spt = reinterpret_cast<float4 *>(smem + lay.offPt);
    uint2 *sslot = reinterpret_cast<uint2 *>(smem + lay.offSlot);
    uint32_t *sm = reinterpret_cast<uint32_t *>(smem + lay.offM);
    uint32_t *scnt = reinterpret_cast<uint32_t *>(smem + lay.offCnt);
    uint32_t *soff = reinterpret_cast<uint32_t *>(smem + lay.offOff);
    uint32_t *scoff = reinterpret_cast<uint32_t *>(smem + lay.offCacheOff);           // [blockM]
    uint32_t *sptL = reinterpret_cast<uint32_t *>(smem + lay.offPtL);                 // [pointCap]
    float4 *sv = reinterpret_cast<float4 *>(smem + lay.offVel);                      // [2 * islandBodies]
    uint32_t *laneL = reinterpret_cast<uint32_t *>(smem + lay.offVel + (size_t)lay.islandBodies * 32);
    uint32_t *unitC = laneL + kIslandUnits * 32;
    uint2 *swb = reinterpret_cast<uint2 *>(unitC + kIslandUnits);                     // [localCap]
    uint32_t *scol = reinterpret_cast<uint32_t *>(swb + lay.localCap);                // [localCap]
    uint32_t *sbody = scol + lay.localCap;                                             // [islandBodies]
    // warm-start cache offsets: the solved point counts in manifold order
    // (every count requested at once: at most kScanPer per thread)
    {
        constexpr int kScanPer = kBlockMaxManifolds / kBlockSolveThreads;
        uint32_t v[kScanPer];
#pragma unroll
        for (int j = 0; j < kScanPer; ++j) {
            const uint32_t i = tid + j * nt;
            v[j] = i < M ? __ldcg(&sb.pcount[i]) : 0u;
        }
#pragma unroll
        for (int j = 0; j < kScanPer; ++j) {
            const uint32_t i = tid + j * nt;
            if (i < M) scoff[i] = v[j];
        }
    }
    if (tid <= kIslandMax) is.classCount[tid] = 0;
    if (tid == 0) is.localUsed = is.pointUsed = is.bodyUsed = 0;
    for (uint32_t i = tid; i < kIslandUnits * 32; i += nt) laneL[i] = kNoLocal;
    for (uint32_t i = tid; i < kIslandUnits; i += nt) unitC[i] = 0;
    // plans in the prepared-point area (the owner's local memory past its
    // capacity; is.plans was cleared before the cluster barrier)
    IslandPlan local;
    IslandPlan *plan = &local;
    if (ownRoot != kNoIsland) {
        const uint32_t planCap = (uint32_t)(((size_t)lay.pointCap * 176) / sizeof(IslandPlan));
        const uint32_t k = atomicAdd(&is.plans, 1u);
        if (k < planCap) plan = reinterpret_cast<IslandPlan *>(spt) + k;
        planIsland(a, sb.islandRec + (size_t)ownRoot * kIslandMax, ownN, *plan);
    }
    IslandPlan &P = *plan;
    __syncthreads();
    uint32_t idx = 0;
    if (ownRoot != kNoIsland) idx = atomicAdd(&is.classCount[P.n], 1u);
    const uint32_t total = blockExclusiveScanArray(scoff, M, cs.solve.scan);  // ends with a barrier
    if (rank == 0 && tid == 0) *newCount = total;
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
    // Owners lay out their islands (local manifolds, points, bodies); slots
    // an island took but could not use are marked empty.
    bool packed = false;
    if (ownRoot != kNoIsland) {
        const uint32_t per = 32 / P.n;
        const uint32_t u = is.classBase[P.n] + idx / per, lane0 = (idx % per) * P.n;
        if (u < kIslandUnits) {
            const uint32_t L0 = atomicAdd(&is.localUsed, P.n);
            const uint32_t P0 = atomicAdd(&is.pointUsed, P.points);
            const uint32_t B0 = atomicAdd(&is.bodyUsed, P.nbody);
            packed = L0 + P.n <= lay.localCap && P0 + P.points <= lay.pointCap && B0 + P.nbody <= lay.islandBodies;
            if (packed) {
                uint32_t o = P0;
                for (uint32_t t = 0; t < P.n; ++t) {
                    const uint32_t L = L0 + t, meta = P.meta[t], pts = planPoints(meta);
                    const uint2 sl = planSlots(meta);
                    sm[L] = P.ks[t];
                    sslot[L] = make_uint2(B0 + sl.x, B0 + sl.y);
                    swb[L] = make_uint2(B0 + t, (B0 + P.nbody) | P.n << 16);
                    scnt[L] = pts;
                    soff[L] = o;
                    scol[L] = planColor(meta);
                    for (uint32_t p = 0; p < pts; ++p) sptL[o + p] = L;
                    o += pts;
                    laneL[u * 32 + lane0 + t] = L;
                }
                for (uint32_t i = 0; i < P.nbody; ++i)
                    sbody[B0 + i] = P.body[i] | ((P.dynMask >> i & 1u) ? 0u : kBodyNotDynamic);
                atomicMax(&unitC[u], P.colors);
            } else {
                for (uint32_t L = L0; L < min(L0 + P.n, lay.localCap); ++L) sm[L] = kNoLocal;
                for (uint32_t o = P0; o < min(P0 + P.points, lay.pointCap); ++o) sptL[o] = kNoLocal;
                for (uint32_t i = B0; i < min(B0 + P.nbody, lay.islandBodies); ++i) sbody[i] = kNoBody;
            }
        }
        if (!packed && plan != &local) local = P;  // the staging overwrites the shared plans
    }
    __syncthreads();
    // Every thread loads its share: a manifold's constants, a point's prepared
    // vectors and impulse, a body's velocities.
    {
        const uint32_t nL = min(is.localUsed, lay.localCap), nP = min(is.pointUsed, lay.pointCap),
                       nB = min(is.bodyUsed, lay.islandBodies);
        const uint32_t n = max(nL, max(nP, nB));
        for (uint32_t j = tid; j < n; j += nt) {
            const uint32_t mL = j < nL ? sm[j] : kNoLocal;
            const uint32_t Lp = j < nP ? sptL[j] : kNoLocal;
            const uint32_t b = j < nB ? sbody[j] : kNoBody;
            float4 pm4, pn4, pt[kPreparedVec4], imp, vl, va;
            if (mL != kNoLocal) {
                pm4 = __ldcg(&sb.pm[mL]);
                pn4 = __ldcg(&sb.pn[mL]);
            }
            if (Lp != kNoLocal) {
                const uint32_t m = sm[Lp], p = j - soff[Lp];
#pragma unroll
                for (int v = 0; v < kPreparedVec4; ++v) pt[v] = __ldcg(&sb.pp[(size_t)(v * 4 + p) * a.mcap + m]);
                imp = __ldcg(&sb.pimp[(size_t)p * a.mcap + m]);
            }
            if (b != kNoBody) {
                vl = ld4(&w.nxt.lin[b & ~kBodyNotDynamic]);
                va = ld4(&w.nxt.ang[b & ~kBodyNotDynamic]);
            }
            if (mL != kNoLocal) {
                spm[j] = pm4;
                spn[j] = pn4;
            }
            if (Lp != kNoLocal) {
#pragma unroll
                for (int v = 0; v < kPreparedVec4; ++v) spt[(size_t)v * lay.pointCap + j] = pt[v];
                spt[(size_t)10 * lay.pointCap + j] = imp;
            }
            if (b != kNoBody) {
                sv[2 * j] = vl;
                sv[2 * j + 1] = va;
            }
        }
    }
    __syncthreads();
    if (stamper) a.st->solverStamp[4] = globalNs();
    // warp units: pass by pass (pass 0: warm start), colour by colour; then
    // each lane's results
    const LocalOnlyPrep pr{a, spm, spn, sm, scnt, soff, spt, lay.pointCap};
    const SharedVel v{sv, sslot};
    for (uint32_t u = warp; u < min(is.units, kIslandUnits); u += nt >> 5) {
        const uint32_t L = laneL[u * 32 + lane], C = unitC[u];
        const uint32_t c = L != kNoLocal ? scol[L] : kNoLocal;
        {
            // warm start: every lane's inverse inertia rows requested at once
            InertiaInRegs wpr{pr};
            if (L != kNoLocal)
#pragma unroll
                for (int j = 0; j < 6; ++j) wpr.r[j] = __ldcg(&sb.pmInertia[(size_t)j * a.mcap + sm[L]]);
            for (uint32_t cc = 0; cc < C; ++cc) {
                if (c == cc) warmStartOne(wpr, L, L, v);
                __syncwarp();
            }
        }
        for (int it = 0; it < a.iterations; ++it)
            for (uint32_t cc = 0; cc < C; ++cc) {
                if (c == cc) solveOne(pr, L, L, v);
                __syncwarp();
            }
        if (L == kNoLocal) continue;
        const uint32_t m = sm[L];
        const uint2 sl = sslot[L], wb = swb[L];
        writeManifoldResult(a, nc, cacheCap, pr, L, m, sbody[sl.x] & ~kBodyNotDynamic,
                            sbody[sl.y] & ~kBodyNotDynamic, scnt[L], scoff[m]);
        for (uint32_t j = wb.x; j < (wb.y & 0xFFFFu); j += wb.y >> 16) {
            const uint32_t b = sbody[j];
            if (b & kBodyNotDynamic) continue;
            st4(&w.nxt.lin[b], sv[2 * j]);
            st4(&w.nxt.ang[b], sv[2 * j + 1]);
        }
    }
    if (ownRoot != kNoIsland && !packed) solveIslandAlone(a, nc, cacheCap, scoff, local);
    __syncthreads();
    if (tid == 0) atomicMax(&a.st->solverStamp[5], globalNs());  // the last rank's
}

// ---------------------------------------------------------- prepare ---
// Prepare, manifold flags and island unions for the cluster kernel, over the
// whole GPU: their scattered loads (some forty sectors per prepared point)
// would queue on the cluster's few SMs.  Items are (manifold, point) pairs
// q = 4 m + p dealt out across the item blocks (item q on block q % B), so
// that a few hundred manifolds still reach every SM; the blocks after them
// take the manifold flags and the unions, one manifold per thread.  Each
// thread requests its manifold's data together with the manifold count
// (indices below the capacities either way).  Nothing is done when the step
// has more than blockM manifolds (the cluster kernel then sends the step to
// the multi-kernel path, and no island link may be left set).
constexpr int kIslPrepThreads = 64;
constexpr uint32_t kIslPrepKeyCap = 2048;  // old cache keys copied to shared memory

__global__ void __launch_bounds__(kIslPrepThreads) k_prepare_islands(SolveArgs a, uint32_t blockM,
                                                                     uint32_t itemBlocks) {
    __shared__ __align__(16) unsigned long long s_keys[kIslPrepKeyCap];
    const uint32_t tid = threadIdx.x;
    if (blockIdx.x == 0 && tid == 0) a.st->solverStamp[0] = globalNs();
    if (blockIdx.x >= itemBlocks) {
        const uint32_t m = (blockIdx.x - itemBlocks) * kIslPrepThreads + tid;
        uint32_t ba = 0, bb = 0, gA = 0, gB = 0;
        if (m < a.mcap) {
            ba = a.mv.bodyA[m];
            bb = a.mv.bodyB[m];
            gA = a.mv.genA[m];
            gB = a.mv.genB[m];
        }
        const uint32_t M = min(*a.count, a.mcap);
        // no unions while the solver skips the island attempt (the links stay 0)
        const bool unite = __ldcg(a.sb.pathHint) == 0u;
        if (M <= blockM && m < M) {
            const uint32_t fl = manifoldFlagsOf(a.w, ba, bb, gA, gB);
            a.sb.dyn[m] = fl;
            if (unite && (fl & (kFlagValid | kFlagDynA | kFlagDynB)) == (kFlagValid | kFlagDynA | kFlagDynB) &&
                !islandUnite(a.sb.islLink, ba, bb))
                atomicOr(&a.st->islandRefused, 1u);
        }
    } else {
        const uint32_t q = tid * itemBlocks + blockIdx.x, m = q >> 2, p = q & 3u;
        PrepItem it{};
        if (m < a.mcap) it = loadPrepItemAt(a, m, p);
        const uint32_t M = min(*a.count, a.mcap), cacheN = *a.oldCount;
        const bool work = M <= blockM && blockIdx.x < 4 * M;  // some item of this block is live
        const bool inShared = cacheN <= kIslPrepKeyCap;
        // a larger cache: every stride-th key in shared memory (two-level search)
        const uint32_t stride = inShared ? 1u : (cacheN + kIslPrepKeyCap - 1) / kIslPrepKeyCap;
        const bool sampled = !inShared && stride <= kCacheSampleStride;
        const uint32_t nS = sampled ? (cacheN + stride - 1) / stride : 0u;
        if (work && sampled)
            for (uint32_t i = tid; i < nS; i += kIslPrepThreads) s_keys[i] = __ldcg(&a.oldCache.key[i * stride]);
        if (work && inShared) {
            // 16-byte loads, every one of a thread's requested before any store
            constexpr uint32_t kPer = kIslPrepKeyCap / 2 / kIslPrepThreads;
            const ulonglong2 *src = reinterpret_cast<const ulonglong2 *>(a.oldCache.key);
            ulonglong2 *dst = reinterpret_cast<ulonglong2 *>(s_keys);
            const uint32_t pairs = cacheN / 2;
            ulonglong2 v[kPer];
#pragma unroll
            for (uint32_t j = 0; j < kPer; ++j) {
                const uint32_t i = tid + j * kIslPrepThreads;
                if (i < pairs) v[j] = __ldcg(&src[i]);
            }
            unsigned long long last = 0;
            if (tid == 0 && (cacheN & 1u)) last = __ldcg(&a.oldCache.key[cacheN - 1]);
#pragma unroll
            for (uint32_t j = 0; j < kPer; ++j) {
                const uint32_t i = tid + j * kIslPrepThreads;
                if (i < pairs) dst[i] = v[j];
            }
            if (tid == 0 && (cacheN & 1u)) s_keys[cacheN - 1] = last;
        }
        __syncthreads();
        if (work && m < M) {
            PrepTally tally;
            if (sampled) {
                const uint2 range = cacheRangeSampled(s_keys, nS, stride, a.oldCache.key, cacheN, it.ia, it.ib);
                prepareItem(a, it, a.oldCache.key, cacheN, tally, &range);
            } else {
                prepareItem(a, it, inShared ? s_keys : a.oldCache.key, cacheN, tally);
            }
            flushPrepTally(a, tally);
        }
    }
    __syncthreads();
    if (tid == 0) atomicMax(&a.st->solverStamp[1], globalNs());  // the last block's end
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
    const bool stamper = rank == 0 && tid == 0;
    auto stamp = [&](int k) {
        if (stamper) a.st->solverStamp[k] = globalNs();
    };
    stamp(2);
    // Manifold um of this thread (consecutive manifolds on other SMs),
    // requested with the counts; k_prepare_islands prepared every manifold,
    // wrote its flags and united the islands.
    const uint32_t um = tid * kClusterRanks + rank;
    uint32_t ufl = 0, ua = 0, ub = 0, upts = 0;
    if (um < a.mcap) {
        ufl = __ldcg(&sb.dyn[um]);
        ua = a.mv.bodyA[um];
        ub = a.mv.bodyB[um];
        upts = __ldcg(&sb.pcount[um]);
    }
    const uint32_t M = min(*a.count, a.mcap);
    if (M > lay.blockM) {  // every rank sees the same count
        if (rank == 0 && tid == 0) atomicOr(&a.st->err, kErrSmallPath);
        return;
    }
    const bool hasU = um < M;
    if (!hasU) ufl = 0;
    // A recent step found islands the island path cannot take (a pile): go
    // straight to the colour-phase path for a few steps (both paths give the
    // same result; this one skips the records and finds).  Every rank reads
    // the hint here, the prepare kernel read it before; rank 0 updates it
    // after the first cluster barrier.
    const uint32_t hint = __ldcg(sb.pathHint);
    uint32_t *link = sb.islLink;   // island links of the bodies (0 between steps)
    uint32_t *isize = sb.islSize;  // manifolds listed at an island root (0 between steps)
    unsigned long long *s_sort = reinterpret_cast<unsigned long long *>(smem);
    uint32_t *s_dyn = reinterpret_cast<uint32_t *>(smem + (size_t)lay.blockM * 8);

    // ---- 1. each solved manifold joins its island's records; the first to
    // join owns the island (M <= blockM <= threads of the cluster: one
    // manifold per thread) ----
    uint32_t ownRoot = kNoIsland;
    bool refuse = hint != 0u;
    if (hasU && !refuse) {
        if (!(ufl & kFlagValid)) {
            // an unsolved manifold that still shapes the colouring: colour-phase path
            if (ufl & (kFlagDynA | kFlagDynB)) refuse = true;
        } else if (!(ufl & (kFlagDynA | kFlagDynB))) {
            refuse = true;  // solved manifold without a dynamic body
        } else {
            const uint32_t r = islandFind(link, (ufl & kFlagDynA) ? ua : ub);
            const uint32_t pos = atomicAdd(&isize[r], 1u);
            if (pos < kIslandMax)
                sb.islandRec[(size_t)r * kIslandMax + pos] = make_uint4(islandRecWord(um, ufl, upts), ua, ub, 0u);
            else refuse = true;
            if (pos == 0) ownRoot = r;
        }
    }
    if (refuse && (hint == 0u || (rank == 0 && tid == 0))) atomicOr(&a.st->islandRefused, 1u);
    if (tid == 0) cs.island.plans = 0;
    // The cluster barriers have release / acquire semantics at cluster scope:
    // what one rank wrote before a barrier, any rank reads after it.
    cluster.sync();
    stamp(3);
    if (rank == 0 && tid == 0) {
        const bool refused = __ldcg(&a.st->islandRefused) != 0u;
        *sb.pathHint = hint ? hint - 1u : (refused ? kPathHintSteps : 0u);
    }
    // Every find is done: the links and the island sizes go back to 0.
    uint32_t ownN = 0;
    if (ownRoot != kNoIsland) {
        ownN = min(__ldcg(&isize[ownRoot]), kIslandMax);
        isize[ownRoot] = 0;
    }
    if (ufl & kFlagDynA) link[ua] = 0;
    if (ufl & kFlagDynB) link[ub] = 0;
    // The island path needs the cache in manifold order (one manifold per body
    // pair): a cache sorted over the solve order needs the order, which only
    // the colour-phase path materialises.
    if (__ldcg(&a.st->islandRefused) == 0 && a.pairOrderCache) {
        // ---- island path ----
        if (um == 0) atomicMax(&a.st->colorRounds, 1u);  // one round when nothing is coloured
        solveIslandsRank(a, nc, cacheCap, newCount, M, rank, lay, smem, ownRoot, ownN, cs, stamper);
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
// afterwards, in the same bytes, the velocity slice, the local manifolds, the
// island path's cache offsets and as many prepared points (176 bytes each) as
// fit.
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
    // phase path) or the islands' body velocities, unit lane maps, colours,
    // bodies and write-back shares (island path)
    l.islandBodies = 2 * l.localCap;
    const size_t islandArea = (size_t)l.islandBodies * 36 + (kIslandUnits * 32 + kIslandUnits) * 4 +
                              (size_t)l.localCap * 12;
    l.offVel = take(std::max<size_t>((size_t)velSlots * 32, islandArea));
    l.offPm = take((size_t)l.localCap * 16);
    l.offPn = take((size_t)l.localCap * 16);
    l.offSlot = take((size_t)l.localCap * 8);
    l.offM = take((size_t)l.localCap * 4);
    l.offCnt = take((size_t)l.localCap * 4);
    l.offOff = take((size_t)l.localCap * 4);
    l.offCacheOff = take((size_t)blockM * 4);
    // prepared points (176 bytes each) and, per point, its local manifold (4)
    l.pointCap = off + 16 < kClusterSmemMax ? (uint32_t)((kClusterSmemMax - off - 16) / 180) : 0u;
    l.offPtL = take((size_t)l.pointCap * 4);
    l.offPt = (uint32_t)off;
    // one rank per SM in any case: take the SM's shared memory
    l.smemBytes = kClusterSmemMax;
    if (off + (size_t)l.pointCap * 176 > kClusterSmemMax) l.pointCap = 0;  // cannot happen: sized above
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
    const uint32_t itemBlocks = (4 * blockM + kIslPrepThreads - 1) / kIslPrepThreads;
    const uint32_t unionBlocks = (blockM + kIslPrepThreads - 1) / kIslPrepThreads;
    k_prepare_islands<<<itemBlocks + unionBlocks, kIslPrepThreads, 0, s>>>(a, blockM, itemBlocks);
    PE_LAUNCHED();
    k_solve_cluster<<<kClusterRanks, kBlockSolveThreads, lay.smemBytes, s>>>(a, newCache, cacheCap, newCacheCount, lay);
    PE_LAUNCHED();
    return true;
}

} // namespace pe
