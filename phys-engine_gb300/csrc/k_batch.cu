// Batched-world step: one persistent kernel per size bucket.  Each thread block
// takes worlds from the bucket's queue (largest first) and runs the whole
// PhysicsWorld::step (src/world/physics_world.cpp:518-782) for one world before
// taking the next:
//   1. integrateVelocity + Aabb::fromCollider for every body
//      (physics_world.cpp:528-551, src/collision/aabb.cpp:8-32);
//   2. SAP: sort by (min.x, index) in shared memory, sweep, pairs sorted to
//      lexicographic order (src/collision/broadphase.cpp:195-291, :18-60);
//   3. narrowphase in pair order with manifolds compacted in that order
//      (physics_world.cpp:645-712);
//   4. the single-block graph-colour solver (colouring, prepare, warm start,
//      velocity iterations, cache rebuild);
//   5. integratePosition / integrateRotation (physics_world.cpp:759-767).
// Stages are separated by __syncthreads; a world never spans two blocks, so no
// block waits on another and no grid barrier is needed.  The device functions
// are the single-world engine's, so each world's results equal that engine's.
#include "batch.h"
#include "pe_bodies.cuh"
#include "pe_narrow.cuh"
#include "pe_solve.cuh"

namespace pe {
namespace {

// Exclusive scan of one value per thread over a block of any multiple of 32
// threads (<= 1024); s needs 33 words.
__device__ __forceinline__ uint32_t scanBlock(uint32_t v, uint32_t &total, uint32_t *s) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t n = __shfl_up_sync(0xffffffffu, incl, o);
        if ((int)lane >= o) incl += n;
    }
    if (lane == 31) s[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const uint32_t x = lane < nw ? s[lane] : 0u;
        uint32_t xi = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t n = __shfl_up_sync(0xffffffffu, xi, o);
            if ((int)lane >= o) xi += n;
        }
        if (lane < nw) s[lane] = xi - x;
        if (lane == 31) s[32] = xi;
    }
    __syncthreads();
    const uint32_t r = s[warp] + incl - v;
    total = s[32];
    __syncthreads();
    return r;
}

__device__ __forceinline__ WorldView worldView(const BatchView &b, const WorldDesc &d) {
    const uint32_t s = d.bodyStart;
    const BodyState &c = b.state[b.parity], &n = b.state[b.parity ^ 1u];
    WorldView w{};
    w.nb = w.nc = d.bodyCount;
    w.cur = BodyState{c.pos + s, c.rot + s, c.lin + s, c.ang + s};
    w.nxt = BodyState{n.pos + s, n.rot + s, n.lin + s, n.ang + s};
    w.force = b.force ? b.force + s : nullptr;
    w.mat = b.mat + s;
    w.iinv = b.iinv + s;
    w.bflags = b.bflags + s;
    w.bgen = b.bgen + s;
    w.cbody = b.cbody + s;
    w.cbgen = b.cbgen + s;
    w.cflags = b.cflags + s;
    w.cshape = b.cshape + s;
    w.clpos = nullptr;
    w.clrot = nullptr;
    w.hullOffset = nullptr;
    w.hullVerts = nullptr;
    w.aabbMin = b.aabbMin + s;
    w.aabbMax = b.aabbMax + s;
    w.gx = b.gx;
    w.gy = b.gy;
    w.gz = b.gz;
    w.dt = b.dt;
    return w;
}

__device__ __forceinline__ ManifoldView manifoldSlice(const ManifoldView &m, uint32_t base) {
    const size_t p = 4ull * base;
    return ManifoldView{m.bodyA + base,          m.genA + base,    m.bodyB + base,   m.genB + base,
                        m.normalFriction + base, m.restitution + base, m.pointCount + base, m.anchorA + p,
                        m.anchorB + p,           m.impulse + p,    m.feature + p};
}

__device__ __forceinline__ CacheView cacheSlice(const CacheView &c, uint32_t base) {
    return CacheView{c.key + base, c.gens + base, c.anchorA + base, c.anchorB + base, c.tangent2 + base};
}

__device__ __forceinline__ SolverBuffers solverSlice(const BatchView &b, const WorldDesc &d, uint32_t wi) {
    SolverBuffers sb{};
    const uint32_t mb = d.mBase;
    sb.mcap = d.mCap;
    sb.bodyBest = b.sb.bodyBest + d.bodyStart;
    sb.bodyUsed = b.sb.bodyUsed + 2ull * d.bodyStart;
    sb.epoch = b.epoch + wi;
    sb.color = b.sb.color + mb;
    sb.dyn = b.sb.dyn + mb;
    sb.colorCount = b.colorCount + (size_t)wi * kMaxColors;
    sb.order = b.sb.order + mb;
    sb.colorStart = b.sb.colorStart + mb;
    sb.pm = b.sb.pm + mb;
    sb.pmInertia = b.sb.pmInertia + 6ull * mb;
    sb.pp = b.sb.pp + (size_t)kPreparedVec4 * 4 * mb;
    sb.pimp = b.sb.pimp + 4ull * mb;
    sb.pn = b.sb.pn + mb;
    sb.pbody = b.sb.pbody + mb;
    sb.pcount = b.sb.pcount + mb;
    return sb;
}

struct BatchShared {
    BlockSolveShared solve;
    uint32_t scan[33];
    uint32_t world;
    uint32_t count;
    unsigned long long xWindow;
};

// One world, all threads of the block.
__device__ __noinline__ void stepWorld(const BatchView &b, uint32_t wi, unsigned long long *smem, BatchShared &sh) {
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    const WorldDesc d = b.worlds[wi];
    DevStats *st = b.stats + wi;
    {
        uint32_t *raw = reinterpret_cast<uint32_t *>(st);
        for (uint32_t i = tid; i < sizeof(DevStats) / 4; i += nt) raw[i] = 0u;
    }
    if (tid == 0) {
        sh.count = 0;
        sh.xWindow = 0;
    }
    const WorldView w = worldView(b, d);
    const uint32_t N = d.bodyCount;
    __syncthreads();

    // 1. velocity, AABB, SAP key
    unsigned long long *keys = smem;
    const uint32_t np = nextPow2(N > 0 ? N : 1);
    for (uint32_t i = tid; i < N; i += nt) {
        const uint32_t f = w.bflags[i];
        V3 lin = f4xyz(w.cur.lin[i]);
        if ((f & kBodyAlive) && !(f & kBodyStatic)) {
            const V3 force = w.force ? f4xyz(w.force[i]) : V3{0.0f, 0.0f, 0.0f};
            lin = integrateVelocity(lin, V3{w.gx, w.gy, w.gz}, force, w.mat[i].x, w.dt);
        }
        w.nxt.lin[i] = make4(lin, 0.0f);
        w.nxt.ang[i] = w.cur.ang[i];
        const uint32_t body = w.cbody[i];
        const Tf t = colliderWorld(w, i, f4xyz(w.cur.pos[body]), f4q(w.cur.rot[body]));
        V3 mn, mx;
        colliderAabb(w, i, t, mn, mx);
        w.aabbMin[i] = make4(mn, 0.0f);
        w.aabbMax[i] = make4(mx, 0.0f);
        keys[i] = ((unsigned long long)orderedFloatKey(mn.x) << 32) | i;
    }
    for (uint32_t i = N + tid; i < np; i += nt) keys[i] = ~0ull;
    __syncthreads();

    // 2. SAP: sort by (min.x, index), sweep with the reference's break and
    // Y/Z test (broadphase.cpp:212-243), then lexicographic pair order.
    blockBitonicSort(keys, np);
    unsigned long long *pk = b.pairKeys + d.pairBase;
    unsigned long long window = 0;
    for (uint32_t i = tid; i < N; i += nt) {
        const uint32_t ia = (uint32_t)keys[i];
        const float4 amn = w.aabbMin[ia], amx = w.aabbMax[ia];
        const uint32_t xk = orderedFloatKey(amx.x);
        uint32_t lo = i + 1, hi = N;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if ((uint32_t)(keys[mid] >> 32) > xk) hi = mid;
            else lo = mid + 1;
        }
        window += lo - i - 1;
        for (uint32_t j = i + 1; j < lo; ++j) {
            const uint32_t jb = (uint32_t)keys[j];
            const float4 bmn = w.aabbMin[jb], bmx = w.aabbMax[jb];
            if (amn.y <= bmx.y && amx.y >= bmn.y && amn.z <= bmx.z && amx.z >= bmn.z) {
                const uint32_t slot = atomicAdd(&sh.count, 1u);
                if (slot < d.pairCap)
                    pk[slot] = ((unsigned long long)min(ia, jb) << 32) | max(ia, jb);
            }
        }
    }
    if (window) atomicAdd(&sh.xWindow, window);
    __syncthreads();
    const uint32_t P = sh.count;
    if (tid == 0) {
        st->inputCount = N;
        st->xWindow = sh.xWindow;
        st->rawPairs = P;
        st->uniquePairs = P;
        st->pairs = P;
    }
    if (P > d.pairCap) {
        if (tid == 0) {
            st->err |= kErrPairCapacity;
            atomicOr(b.batchErr, kErrPairCapacity);
        }
        __syncthreads();
        return;
    }
    const uint32_t pp = nextPow2(P > 0 ? P : 1);
    for (uint32_t i = P + tid; i < pp; i += nt) pk[i] = ~0ull;
    __syncthreads();
    blockBitonicSort(pk, pp);

    // 3. narrowphase in pair order
    const ManifoldView mv = manifoldSlice(b.mv, d.mBase);
    uint32_t running = 0;
    for (uint32_t t0 = 0; t0 < P; t0 += nt) {
        const uint32_t p = t0 + tid;
        LocalManifold lm;
        lm.count = 0;
        bool hit = false;
        uint32_t ca = 0, cb = 0, ba = 0, bb = 0, category = 0;
        float restitution = 0.0f, friction = 0.0f;
        if (p < P) {
            const unsigned long long key = pk[p];
            ca = (uint32_t)(key >> 32);
            cb = (uint32_t)key;
            ba = w.cbody[ca];
            bb = w.cbody[cb];
            bool epaFailed;
            hit = narrowphasePair(w, ca, cb, ba, bb, lm, restitution, friction, category, epaFailed);
            if (epaFailed) atomicAdd(&st->epaFailures, 1ull);
            aggregatedCount(st->npCandidates, category);
            if (hit) aggregatedCount(st->npContacts, category);
        }
        uint32_t total;
        const uint32_t m = running + scanBlock(hit ? 1u : 0u, total, sh.scan);
        if (hit) {
            if (m < d.mCap) storeManifold(mv, m, w, ca, cb, ba, bb, lm, restitution, friction);
            atomicAdd(&st->points, lm.count);
        }
        running += total;
    }
    if (tid == 0) st->manifolds = running;
    if (running > d.mCap) {
        if (tid == 0) {
            st->err |= kErrManifoldCapacity;
            atomicOr(b.batchErr, kErrManifoldCapacity);
        }
        __syncthreads();
        return;
    }
    __syncthreads();

    // 4. contact solve (graph-colour order)
    SolveArgs a;
    a.w = w;
    a.mv = mv;
    a.sb = solverSlice(b, d, wi);
    a.oldCache = cacheSlice(b.cache[b.parity], d.cacheBase);
    a.oldCount = b.cacheCount + (size_t)b.parity * b.worldCount + wi;
    a.st = st;
    a.mcap = d.mCap;
    a.iterations = b.iterations;
    a.pairOrderCache = true;  // collider i is body i in every batched world
    a.count = &st->manifolds;
    const CacheView nc = cacheSlice(b.cache[b.parity ^ 1u], d.cacheBase);
    uint32_t *newCount = b.cacheCount + (size_t)(b.parity ^ 1u) * b.worldCount + wi;
    solveBlock(a, nc, d.cacheCap, newCount, 0, b.maxM, smem, reinterpret_cast<uint32_t *>(smem + b.maxM), sh.solve);
    __syncthreads();

    // 5. pose
    for (uint32_t i = tid; i < N; i += nt) {
        const uint32_t f = w.bflags[i];
        float4 p4 = w.cur.pos[i], q4 = w.cur.rot[i];
        if ((f & kBodyAlive) && !(f & kBodyStatic)) {
            V3 pos = f4xyz(p4);
            Q rot = f4q(q4);
            integratePose(pos, rot, f4xyz(ld4(&w.nxt.lin[i])), f4xyz(ld4(&w.nxt.ang[i])), w.dt);
            p4 = make4(pos, 0.0f);
            q4 = make4(rot);
        }
        w.nxt.pos[i] = p4;
        w.nxt.rot[i] = q4;
    }
    __syncthreads();
    if (tid == 0 && st->err) atomicOr(b.batchErr, st->err);
}

template <int T, int B> __global__ void __launch_bounds__(T, B) k_batch_step(BatchView b) {
    extern __shared__ unsigned long long s_dynamic[];
    __shared__ BatchShared sh;
    for (;;) {
        if (threadIdx.x == 0) sh.world = atomicAdd(b.queueHead, 1u);
        __syncthreads();
        const uint32_t q = sh.world;
        __syncthreads();
        if (q >= b.queueLen) return;
        stepWorld(b, b.queue[q], s_dynamic, sh);
    }
}

using BatchKernel = void (*)(BatchView);
// Must list the variants of kBatchVariants in the same order.
const BatchKernel kKernels[] = {k_batch_step<128, 1>, k_batch_step<128, 4>, k_batch_step<256, 1>,
                                k_batch_step<256, 2>, k_batch_step<512, 1>};
static_assert(sizeof(kKernels) / sizeof(kKernels[0]) == kBatchVariantCount, "one kernel per variant");

} // namespace

size_t batchSharedBytes(uint32_t maxN, uint32_t maxM) {
    size_t np = 1;
    while (np < maxN) np <<= 1;
    const size_t sap = 8ull * np;
    const size_t solve = 12ull * maxM;
    return sap > solve ? sap : solve;
}

uint32_t batchMaxBlocks(int variant, size_t smem) {
    if (variant < 0 || variant >= kBatchVariantCount) throw std::invalid_argument("unknown batch kernel variant");
    int dev = 0, sms = 0, per = 0;
    PE_CHECK(cudaGetDevice(&dev));
    PE_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // The limit is per kernel: raise it, never lower it below what another
    // bucket launching the same variant needs.
    cudaFuncAttributes attr;
    PE_CHECK(cudaFuncGetAttributes(&attr, kKernels[variant]));
    if ((size_t)attr.maxDynamicSharedSizeBytes < smem)
        PE_CHECK(cudaFuncSetAttribute(kKernels[variant], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    PE_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kKernels[variant], kBatchVariants[variant].threads,
                                                           smem));
    if (per < 1) throw std::runtime_error("batch kernel does not fit on an SM with this shared memory");
    return (uint32_t)(per * sms);
}

void launchBatchBucket(const BatchView &b, int variant, uint32_t blocks, cudaStream_t s) {
    if (variant < 0 || variant >= kBatchVariantCount) throw std::invalid_argument("unknown batch kernel variant");
    if (!blocks || !b.queueLen) return;
    const size_t smem = batchSharedBytes(b.maxN, b.maxM);
    kKernels[variant]<<<blocks, kBatchVariants[variant].threads, smem, s>>>(b);
    PE_LAUNCHED();
}

} // namespace pe
