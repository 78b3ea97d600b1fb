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

struct ClusterShared {
    BlockSolveShared solve;
    uint32_t start[kMaxColors + 1];   // colour ranges of the solve order
    uint32_t lstart[kMaxColors + 1];  // colour ranges of this rank's local manifolds
    uint32_t colors, slots, slotted, manifolds;
};

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
        if (tid == 0) {
            sb.counters[0] = slotted ? cs.solve.slots : 0u;
            sb.counters[1] = slotted ? 1u : 0u;
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
    const uint32_t C = cs.colors, Lr = cs.lstart[C], S = cs.slots;
    float4 *sv = reinterpret_cast<float4 *>(smem + lay.offVel);
    float4 *spm = reinterpret_cast<float4 *>(smem + lay.offPm);
    float4 *spn = reinterpret_cast<float4 *>(smem + lay.offPn);
    float4 *spt = reinterpret_cast<float4 *>(smem + lay.offPt);
    uint2 *sslot = reinterpret_cast<uint2 *>(smem + lay.offSlot);
    uint32_t *sm = reinterpret_cast<uint32_t *>(smem + lay.offM);
    uint32_t *scnt = reinterpret_cast<uint32_t *>(smem + lay.offCnt);
    uint32_t *soff = reinterpret_cast<uint32_t *>(smem + lay.offOff);
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
    if (!a.pairOrderCache) {
        if (rank != 0) return;
        solveBlockCache(a, nc, cacheCap, newCount, M, s_sort, s_dyn, cs.solve);
        return;
    }
    // Cache in manifold order (one manifold per body pair, pairs in body
    // order): every rank scans the point counts and writes its interleaved
    // share of the manifolds' entries (as solveBlockCache does on one block).
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
    l.offVel = take((size_t)velSlots * 32);
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
