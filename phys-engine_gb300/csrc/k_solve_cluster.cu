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
// never written, so they join nothing).  Islands share no written state: one
// thread can run every sweep of a small island on its own, in the island's
// (colour, index) order, with no barrier at all; that is the order the
// colour-phase sweeps give every body of the island.
constexpr uint32_t kIslandMax = 8;           // larger islands take the colour-phase path
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

struct ClusterShared {
    BlockSolveShared solve;
    uint32_t start[kMaxColors + 1];   // colour ranges of the solve order
    uint32_t lstart[kMaxColors + 1];  // colour ranges of this rank's local manifolds
    uint32_t colors, slots, slotted, islands;
    uint32_t rankManifolds[kClusterRanks];
    uint32_t islandFail;
};

// Islands of the ordered manifolds (rank 0, after the front): per root slot
// the range of its manifolds (solve indices, in no particular order) in
// sb.compList.  work: 3 * cap words (the front's velocity area); rootK: M
// words.  Returns whether every island is small, all slots fit the per-rank
// velocity arrays and every rank's islands fit its local manifold capacity.
__device__ bool islandFront(const SolveArgs &a, uint32_t M, uint32_t S, const uint32_t *order, const uint2 *slotK,
                            uint32_t *work, uint32_t cap, uint32_t *rootK, const ClusterSolveLayout &lay,
                            ClusterShared &cs) {
    const SolverBuffers &sb = a.sb;
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    uint32_t *parent = work, *cnt = work + cap, *cur = work + 2 * cap;
    for (uint32_t sl = tid; sl < S; sl += nt) {
        parent[sl] = sl;
        cnt[sl] = 0;
    }
    if (tid < kClusterRanks) cs.rankManifolds[tid] = 0;
    if (tid == 0) cs.islandFail = S > lay.islandSlots ? 1u : 0u;
    __syncthreads();
    for (uint32_t k = tid; k < M; k += nt) {
        const uint32_t fl = __ldcg(&sb.dyn[order[k]]);
        rootK[k] = fl;
        if ((fl & (kFlagValid | kFlagDynA | kFlagDynB)) == (kFlagValid | kFlagDynA | kFlagDynB))
            if (!islandUnite(parent, slotK[k].x, slotK[k].y)) cs.islandFail = 1;
    }
    __syncthreads();
    for (uint32_t sl = tid; sl < S; sl += nt) parent[sl] = islandFind(parent, sl);
    __syncthreads();
    for (uint32_t k = tid; k < M; k += nt) {
        const uint32_t fl = rootK[k];
        uint32_t r = kNoIsland;
        if (fl & kFlagValid) {
            if (fl & kFlagDynA) r = parent[slotK[k].x];
            else if (fl & kFlagDynB) r = parent[slotK[k].y];
            else cs.islandFail = 1;  // solved manifold without a dynamic body: colour-phase path
        }
        rootK[k] = r;
        if (r != kNoIsland) atomicAdd(&cnt[r], 1u);
    }
    __syncthreads();
    for (uint32_t sl = tid; sl < S; sl += nt) {
        const uint32_t c = cnt[sl];
        if (c > kIslandMax) cs.islandFail = 1;
        if (c) atomicAdd(&cs.rankManifolds[sl % kClusterRanks], c);
        cur[sl] = c;
    }
    __syncthreads();
    blockExclusiveScanArray(cur, S, cs.solve.scan);
    for (uint32_t sl = tid; sl < S; sl += nt) sb.compRange[sl] = make_uint2(cur[sl], cnt[sl]);
    if (tid < kClusterRanks && cs.rankManifolds[tid] > lay.localCap) cs.islandFail = 1;
    __syncthreads();
    for (uint32_t k = tid; k < M; k += nt) {
        const uint32_t r = rootK[k];
        if (r != kNoIsland) sb.compList[atomicAdd(&cur[r], 1u)] = k;
    }
    __syncthreads();
    return cs.islandFail == 0;
}

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
        s_cnt[i] = (__ldcg(&sb.dyn[i]) & kFlagValid) ? a.mv.pointCount[i] : 0u;
    __syncthreads();
    const uint32_t total = blockExclusiveScanArray(s_cnt, M, cs.solve.scan);
    for (uint32_t i = rank + kClusterRanks * tid; i < M; i += kClusterRanks * nt) {
        const uint32_t cnt = (i + 1 < M ? s_cnt[i + 1] : total) - s_cnt[i];
        cacheWriteManifold(a, nc, cacheCap, i, s_cnt[i], cnt);
    }
    if (rank == 0 && tid == 0) *newCount = total;
}

// Island sweeps (all ranks): rank r takes the islands whose root slot is r
// modulo R, one thread per island; every rank holds the velocities of all
// staged bodies (slot-indexed) and its islands' prepared data.
__device__ void solveIslands(const SolveArgs &a, const ClusterSolveLayout &lay, uint32_t rank, uint32_t S, float4 *sv,
                             float4 *spm, float4 *spn, float4 *spt, uint2 *sslot, uint32_t *sm, uint32_t *scnt,
                             uint32_t *soff, uint32_t *scan, ClusterShared &cs) {
    const SolverBuffers &sb = a.sb;
    const WorldView &w = a.w;
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    for (uint32_t sl = tid; sl < S; sl += nt) {
        const uint32_t b = __ldcg(&sb.stageBody[sl]);
        sv[2 * sl] = ld4(&w.nxt.lin[b]);
        sv[2 * sl + 1] = ld4(&w.nxt.ang[b]);
    }
    // local manifold ranges: a block scan of each thread's island sizes
    uint32_t mine = 0;
    for (uint32_t r = rank + kClusterRanks * tid; r < S; r += kClusterRanks * nt) mine += __ldcg(&sb.compRange[r]).y;
    scan[tid] = mine;
    __syncthreads();
    blockExclusiveScanArray(scan, nt, cs.solve.scan);
    const uint32_t base = scan[tid];
    __syncthreads();
    // each island's manifolds in solve order, then their data
    uint32_t L = base, points = 0;
    for (uint32_t r = rank + kClusterRanks * tid; r < S; r += kClusterRanks * nt) {
        const uint2 rng = __ldcg(&sb.compRange[r]);
        if (!rng.y) continue;
        uint32_t ks[kIslandMax];
        const uint32_t n = min(rng.y, kIslandMax);
        for (uint32_t j = 0; j < n; ++j) {
            const uint32_t k = __ldcg(&sb.compList[rng.x + j]);
            uint32_t i = j;
            for (; i > 0 && ks[i - 1] > k; --i) ks[i] = ks[i - 1];
            ks[i] = k;
        }
        for (uint32_t j = 0; j < n; ++j, ++L) {
            const uint32_t k = ks[j], m = __ldcg(&sb.order[k]);
            sm[L] = m;
            sslot[L] = __ldcg(&sb.stageSlot[k]);
            spm[L] = __ldcg(&sb.pm[m]);
            spn[L] = __ldcg(&sb.pn[m]);
            scnt[L] = __ldcg(&sb.pcount[m]);
            points += scnt[L];
        }
    }
    const uint32_t end = L;
    scan[tid] = points;
    __syncthreads();
    blockExclusiveScanArray(scan, nt, cs.solve.scan);
    uint32_t o = scan[tid];
    for (uint32_t L2 = base; L2 < end; ++L2) {
        const uint32_t n = scnt[L2], m = sm[L2];
        if (o + n > lay.pointCap) {  // past the local capacity: the solver arrays
            soff[L2] = kNoLocal;
            continue;
        }
        soff[L2] = o;
        for (uint32_t p = 0; p < n; ++p) {
#pragma unroll
            for (int v = 0; v < kPreparedVec4; ++v)
                spt[(size_t)v * lay.pointCap + o + p] = __ldcg(&sb.pp[(size_t)(v * 4 + p) * a.mcap + m]);
            spt[(size_t)10 * lay.pointCap + o + p] = __ldcg(&sb.pimp[(size_t)p * a.mcap + m]);
        }
        o += n;
    }
    __syncthreads();  // velocities of every slot loaded
    // sweeps: every island on its own thread, pass by pass (pass 0: warm start)
    const LocalPrep pr{a, spm, spn, sm, scnt, soff, spt, lay.pointCap};
    const SharedVel vel{sv, sslot};
    uint32_t b0 = base;
    for (uint32_t r = rank + kClusterRanks * tid; r < S; r += kClusterRanks * nt) {
        const uint32_t n = min(__ldcg(&sb.compRange[r]).y, kIslandMax);
        if (!n) continue;
        bool local = true;
        for (uint32_t j = 0; j < n; ++j) local = local && soff[b0 + j] != kNoLocal;
        if (local) {
            const LocalOnlyPrep lp{a, spm, spn, sm, scnt, soff, spt, lay.pointCap};
            for (uint32_t j = 0; j < n; ++j) warmStartOne(lp, b0 + j, b0 + j, vel);
            for (int it = 0; it < a.iterations; ++it)
                for (uint32_t j = 0; j < n; ++j) solveOne(lp, b0 + j, b0 + j, vel);
        } else {
            for (uint32_t j = 0; j < n; ++j) warmStartOne(pr, b0 + j, b0 + j, vel);
            for (int it = 0; it < a.iterations; ++it)
                for (uint32_t j = 0; j < n; ++j) solveOne(pr, b0 + j, b0 + j, vel);
        }
        b0 += n;
    }
    // velocities of the islands' dynamic bodies and the impulses back
    for (uint32_t L2 = base; L2 < end; ++L2) {
        const float4 pm = spm[L2];
        const uint2 sl = sslot[L2];
        if (pm.y == 0.0f) {
            const uint32_t b = __ldcg(&sb.stageBody[sl.x]);
            st4(&w.nxt.lin[b], sv[2 * sl.x]);
            st4(&w.nxt.ang[b], sv[2 * sl.x + 1]);
        }
        if (pm.w == 0.0f) {
            const uint32_t b = __ldcg(&sb.stageBody[sl.y]);
            st4(&w.nxt.lin[b], sv[2 * sl.y]);
            st4(&w.nxt.ang[b], sv[2 * sl.y + 1]);
        }
        const uint32_t m = sm[L2], n = scnt[L2];
        for (uint32_t p = 0; p < n; ++p) {
            float4 imp = pr.imp(p, L2);
            imp.w = 0.0f;
            a.mv.impulse[4 * m + p] = imp;
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
    const uint32_t M = min(a.st->manifolds, a.mcap);
    if (M > lay.blockM) {  // every rank sees the same count
        if (rank == 0 && tid == 0) atomicOr(&a.st->err, kErrSmallPath);
        return;
    }

    // ---- 0. ranks 1..: the manifold flags the front reads ----
    // (manifolds interleaved over the ranks: a few hundred manifolds spread
    // over all seven SMs, whose scattered loads are what costs time)
    const uint32_t pfirst = rank - 1 + (kClusterRanks - 1) * tid, pstride = (kClusterRanks - 1) * nt;
    if (rank != 0)
        for (uint32_t m = pfirst; m < M; m += pstride) sb.dyn[m] = manifoldFlags(a, m);
    __threadfence();
    cluster.sync();

    // ---- 1. rank 0: slots, colours, order; ranks 1..: prepare ----
    unsigned long long *s_sort = reinterpret_cast<unsigned long long *>(smem);
    uint32_t *s_dyn = reinterpret_cast<uint32_t *>(smem + (size_t)lay.blockM * 8);
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
        bool islands = false;
        if (slotted)
            islands = islandFront(a, M, cs.solve.slots, s_dyn, vs.slot, reinterpret_cast<uint32_t *>(vs.v), vs.cap,
                                  reinterpret_cast<uint32_t *>(s_sort), lay, cs);
        if (tid == 0) {
            sb.counters[0] = slotted ? cs.solve.slots : 0u;
            sb.counters[1] = slotted ? 1u : 0u;
            sb.counters[2] = islands ? 1u : 0u;
        }
    } else {
        // old cache keys in this rank's shared memory when they fit
        const uint32_t cacheN = *a.oldCount;
        const bool keysInShared = (size_t)cacheN * 8 <= lay.smemBytes;
        if (keysInShared)
            for (uint32_t i = tid; i < cacheN; i += nt) s_sort[i] = a.oldCache.key[i];
        __syncthreads();
        prepareRange(a, pfirst, pstride, M, keysInShared ? s_sort : nullptr);
    }
    __threadfence();
    cluster.sync();

    // ---- 2. this rank's share of every colour and of the staging slots ----
    if (tid == 0) {
        cs.slotted = __ldcg(&sb.counters[1]);
        cs.slots = __ldcg(&sb.counters[0]);
        cs.islands = __ldcg(&sb.counters[2]);
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
    if (cs.islands) {
        solveIslands(a, lay, rank, cs.slots, sv, spm, spn, spt, sslot, sm, scnt, soff,
                     reinterpret_cast<uint32_t *>(smem + lay.offScan), cs);
        __threadfence();
        cluster.sync();
        solveClusterCache(a, nc, cacheCap, newCount, M, rank, smem, s_sort, s_dyn, cs);
        return;
    }
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
    solveClusterCache(a, nc, cacheCap, newCount, M, rank, smem, s_sort, s_dyn, cs);
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
    // the velocity area holds this rank's slice (colour-phase path) or every
    // staged slot (island path)
    l.islandSlots = stageSlots < 2048u ? stageSlots : 2048u;
    l.offVel = take((size_t)(velSlots > l.islandSlots ? velSlots : l.islandSlots) * 32);
    l.offScan = take((size_t)kBlockSolveThreads * 4);
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
