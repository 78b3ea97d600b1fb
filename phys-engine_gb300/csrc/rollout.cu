// GPU differentiable rollout (rollout.h): device layout, the forward and the
// adjoint kernels, and the host driver.
#include <algorithm>
#include <cstring>
#include <stdexcept>
#include <string>

#include "ad_world.cuh"
#include "rollout.h"

namespace pe {
namespace {

using namespace ad;
using F = float;

__host__ __device__ constexpr size_t align16(size_t v) { return (v + 15) & ~size_t(15); }

// Byte offsets inside one world's slot of the arena.
struct Layout {
    // snapshots (checkpoints first, then the segment's states)
    size_t snap0, snapStride;
    size_t sState, sCount, sKey, sA, sB, sLam;  // within a snapshot
    // step scratch (one per step of a segment)
    size_t scr0, scrStride;
    size_t aabb, pairA, pairB, mA, mB, mCount, mFeature, mNormal, mMu, mRest, mAnchorA, mAnchorB, mDepth, color,
        order, sortKeys, bodyUsed, colorStart, pp, pm, lam, lamInit, match, tape, cacheSrc, counts;
    // adjoints
    size_t ax, aq, av, aw, alam, app, apm, an, amuM, arestM, acache, amass, amu, arest, v1v, v1w;
    // broadphase sort buffers, shared by the steps (not part of any record)
    size_t bpEntries, bpPairs;
    size_t stride;
};

__host__ __device__ Layout makeLayout(uint32_t nMax, uint32_t maxPairs, uint32_t maxM, int iterations, uint32_t nSnap,
                                      uint32_t nScr) {
    Layout L{};
    const uint32_t cap = 4 * maxM;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o = align16(o + bytes);
        return at;
    };
    L.sState = take(sizeof(F) * 13 * nMax);
    L.sCount = take(sizeof(uint32_t));
    L.sKey = take(sizeof(unsigned long long) * cap);
    L.sA = take(sizeof(F) * 3 * cap);
    L.sB = take(sizeof(F) * 3 * cap);
    L.sLam = take(sizeof(F) * 3 * cap);
    L.snapStride = o;
    o = 0;
    L.aabb = take(sizeof(F) * 6 * nMax);
    L.pairA = take(4ull * maxPairs);
    L.pairB = take(4ull * maxPairs);
    L.mA = take(4ull * maxM);
    L.mB = take(4ull * maxM);
    L.mCount = take(4ull * maxM);
    L.mFeature = take(16ull * maxM);
    L.mNormal = take(sizeof(F) * 3 * maxM);
    L.mMu = take(sizeof(F) * maxM);
    L.mRest = take(sizeof(F) * maxM);
    L.mAnchorA = take(sizeof(F) * 12 * maxM);
    L.mAnchorB = take(sizeof(F) * 12 * maxM);
    L.mDepth = take(sizeof(F) * 4 * maxM);
    L.color = take(4ull * maxM);
    L.order = take(4ull * maxM);
    L.sortKeys = take(8ull * maxM);
    L.bodyUsed = take(16ull * nMax);
    L.colorStart = take(4ull * (maxM + 1));
    L.pp = take(sizeof(F) * 4 * maxM * kPreparedScalars);
    L.pm = take(sizeof(F) * maxM * kPmScalars);
    L.lam = take(sizeof(F) * 12 * maxM);
    L.lamInit = take(sizeof(F) * 12 * maxM);
    L.match = take(16ull * maxM);
    L.tape = take(sizeof(F) * (size_t)(iterations > 0 ? iterations : 1) * maxM * kTapeScalars);
    L.cacheSrc = take(4ull * cap);
    L.counts = take(16);
    L.scrStride = o;
    o = 0;
    L.snap0 = take(L.snapStride * nSnap);
    L.scr0 = take(L.scrStride * nScr);
    L.ax = take(sizeof(F) * 3 * nMax);
    L.aq = take(sizeof(F) * 4 * nMax);
    L.av = take(sizeof(F) * 3 * nMax);
    L.aw = take(sizeof(F) * 3 * nMax);
    L.alam = take(sizeof(F) * 12 * maxM);
    L.app = take(sizeof(F) * 4 * maxM * kPreparedScalars);
    L.apm = take(sizeof(F) * maxM * kPmScalars);
    L.an = take(sizeof(F) * 3 * maxM);
    L.amuM = take(sizeof(F) * maxM);
    L.arestM = take(sizeof(F) * maxM);
    L.acache = take(sizeof(F) * 3 * cap);
    L.amass = take(sizeof(F) * nMax);
    L.amu = take(sizeof(F) * nMax);
    L.arest = take(sizeof(F) * nMax);
    L.v1v = take(sizeof(F) * 3 * nMax);
    L.v1w = take(sizeof(F) * 3 * nMax);
    L.bpEntries = take(8ull * ad::nextPow2u(nMax > 0 ? nMax : 1));
    L.bpPairs = take(8ull * ad::nextPow2u(maxPairs > 0 ? maxPairs : 1));
    L.stride = o;
    return L;
}

// Capacities of a world of n bodies: candidate pairs, manifolds (a power of
// two), and its slot of the arena, sized for those.
__host__ __device__ inline uint32_t worldMaxPairs(uint32_t n) { return 8 * n + 64; }
// quarterPerBody: manifold capacity in quarter manifolds per body (8 = two
// per body, enough for boxes resting on one another).
__host__ __device__ inline uint32_t worldMaxManifolds(uint32_t n, uint32_t quarterPerBody) {
    const uint64_t need = ((uint64_t)quarterPerBody * n + 3) / 4 + 32;
    uint32_t m = 1;
    while (m < need) m <<= 1;
    return m;
}

struct Args {
    unsigned char *arena;
    const unsigned long long *worldOff;  // byte offset of each world's slot in the arena
    const uint32_t *order;               // worlds in the order blocks take them (largest first)
    const uint32_t *bodyStart;           // worlds + 1
    const uint8_t *shape, *isStatic;
    const F *dims, *iinv, *mass, *mu, *rest;
    uint32_t worlds, steps, ckEvery, nCk, quarterPerBody;
    int iterations;
    F gx, gy, gz, dt;
    uint32_t *queueHead;
    uint32_t *err;  // per world
};

// One world's slot: its layout (sized by its own body count) and base address.
struct Slot {
    Layout L;
    unsigned char *base;
    uint32_t maxPairs, maxM;
};
__device__ __forceinline__ Slot slotOf(const Args &a, uint32_t w) {
    const uint32_t n = a.bodyStart[w + 1] - a.bodyStart[w];
    Slot s;
    s.maxPairs = worldMaxPairs(n);
    s.maxM = worldMaxManifolds(n, a.quarterPerBody);
    s.L = makeLayout(n, s.maxPairs, s.maxM, a.iterations, a.nCk + a.ckEvery + 1, a.ckEvery);
    s.base = a.arena + a.worldOff[w];
    return s;
}

template <class P> __device__ __forceinline__ P *at(unsigned char *base, size_t off) {
    return reinterpret_cast<P *>(base + off);
}

struct Snap {
    ad::StateView<F> s;
    ad::CacheView<F> c;
};
__device__ __forceinline__ Snap snapshot(const Slot &ws, uint32_t j, uint32_t n) {
    unsigned char *p = ws.base + ws.L.snap0 + ws.L.snapStride * j;
    F *st = at<F>(p, ws.L.sState);
    Snap r;
    r.s = ad::StateView<F>{st, st + 3 * n, st + 7 * n, st + 10 * n};
    r.c = ad::CacheView<F>{at<uint32_t>(p, ws.L.sCount), at<unsigned long long>(p, ws.L.sKey), at<F>(p, ws.L.sA),
                       at<F>(p, ws.L.sB), at<F>(p, ws.L.sLam), 4 * ws.maxM};
    return r;
}
__device__ __forceinline__ StepScratch<F> scratch(const Slot &ws, uint32_t j) {
    unsigned char *p = ws.base + ws.L.scr0 + ws.L.scrStride * j;
    const Layout &L = ws.L;
    StepScratch<F> s;
    s.aabb = at<F>(p, L.aabb);
    s.pairA = at<uint32_t>(p, L.pairA);
    s.pairB = at<uint32_t>(p, L.pairB);
    s.mA = at<uint32_t>(p, L.mA);
    s.mB = at<uint32_t>(p, L.mB);
    s.mCount = at<uint32_t>(p, L.mCount);
    s.mFeature = at<uint32_t>(p, L.mFeature);
    s.mNormal = at<F>(p, L.mNormal);
    s.mMu = at<F>(p, L.mMu);
    s.mRest = at<F>(p, L.mRest);
    s.mAnchorA = at<F>(p, L.mAnchorA);
    s.mAnchorB = at<F>(p, L.mAnchorB);
    s.mDepth = at<F>(p, L.mDepth);
    s.color = at<uint32_t>(p, L.color);
    s.order = at<uint32_t>(p, L.order);
    s.sortKeys = at<unsigned long long>(p, L.sortKeys);
    s.bodyUsed = at<unsigned long long>(p, L.bodyUsed);
    s.colorStart = at<uint32_t>(p, L.colorStart);
    s.pp = at<F>(p, L.pp);
    s.pm = at<F>(p, L.pm);
    s.lam = at<F>(p, L.lam);
    s.lamInit = at<F>(p, L.lamInit);
    s.match = at<int32_t>(p, L.match);
    s.tape = at<F>(p, L.tape);
    s.cacheSrc = at<uint32_t>(p, L.cacheSrc);
    s.counts = at<uint32_t>(p, L.counts);
    s.bpEntries = at<unsigned long long>(ws.base, L.bpEntries);
    s.bpPairs = at<unsigned long long>(ws.base, L.bpPairs);
    return s;
}

__device__ __forceinline__ WorldParams<F> params(const Args &a, uint32_t w, const Slot &ws) {
    const uint32_t b = a.bodyStart[w];
    WorldParams<F> W;
    W.n = a.bodyStart[w + 1] - b;
    W.shape = a.shape + b;
    W.isStatic = a.isStatic + b;
    W.dims = a.dims + 3 * b;
    W.iinv = a.iinv + 3 * b;
    W.mass = a.mass + b;
    W.mu = a.mu + b;
    W.rest = a.rest + b;
    W.gx = a.gx;
    W.gy = a.gy;
    W.gz = a.gz;
    W.dt = a.dt;
    W.iterations = a.iterations;
    W.maxPairs = ws.maxPairs;
    W.maxManifolds = ws.maxM;
    return W;
}

__device__ void copySnap(const Snap &from, const Snap &to, uint32_t n) {
    for (uint32_t i = threadIdx.x; i < 13 * n; i += blockDim.x) to.s.x[i] = from.s.x[i];
    const uint32_t c = *from.c.count;
    for (uint32_t e = threadIdx.x; e < c; e += blockDim.x) {
        to.c.key[e] = from.c.key[e];
        for (int j = 0; j < 3; ++j) {
            to.c.anchorA[3 * e + j] = from.c.anchorA[3 * e + j];
            to.c.anchorB[3 * e + j] = from.c.anchorB[3 * e + j];
            to.c.lam[3 * e + j] = from.c.lam[3 * e + j];
        }
    }
    if (threadIdx.x == 0) *to.c.count = c;
    __syncthreads();
}

__device__ __forceinline__ uint32_t nextWorld(const Args &a) {
    __shared__ uint32_t s_w;
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t i = atomicAdd(a.queueHead, 1u);
        s_w = i < a.worlds ? a.order[i] : a.worlds;
    }
    __syncthreads();
    return s_w;
}

// Forward: steps every world, keeps a checkpoint every ckEvery steps (and the
// final state), writes the final state.
// Four blocks per SM (at most 128 registers a thread): the forward pass is
// latency-bound, and the fourth resident world measured 102 -> 83 ms on
// 1,024 worlds of 64 boxes (the adjoint keeps its registers: capping it
// spilled and doubled its time).
__global__ void __launch_bounds__(128, 4) k_rollout_forward(Args a, const F *x0, const F *q0, const F *v0, const F *w0,
                                                       F *xT, F *qT, F *vT, F *wT) {
    for (;;) {
        const uint32_t w = nextWorld(a);
        if (w >= a.worlds) return;
        const Slot ws = slotOf(a, w);
        const WorldParams<F> W = params(a, w, ws);
        const uint32_t n = W.n, b = a.bodyStart[w];
        Snap ck0 = snapshot(ws, 0, n);
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            for (int j = 0; j < 3; ++j) {
                ck0.s.x[3 * i + j] = x0[3 * (b + i) + j];
                ck0.s.v[3 * i + j] = v0[3 * (b + i) + j];
                ck0.s.w[3 * i + j] = w0[3 * (b + i) + j];
            }
            for (int j = 0; j < 4; ++j) ck0.s.q[4 * i + j] = q0[4 * (b + i) + j];
        }
        if (threadIdx.x == 0) *ck0.c.count = 0;
        __syncthreads();
        Snap cur = ck0;
        bool failed = false;
        const StepScratch<F> sc = scratch(ws, 0);
        for (uint32_t t = 0; t < a.steps && !failed; ++t) {
            Snap out = snapshot(ws, a.nCk + (t & 1), n);
            forwardStep<F, BlockTeam>(W, cur.s, cur.c, out.s, out.c, sc, false);
            if (sc.counts[3]) {
                if (threadIdx.x == 0) atomicOr(&a.err[w], sc.counts[3]);
                failed = true;
                break;
            }
            const uint32_t s = t + 1;
            if (s % a.ckEvery == 0 || s == a.steps) {
                const Snap ck = snapshot(ws, (s + a.ckEvery - 1) / a.ckEvery, n);
                copySnap(out, ck, n);
                cur = ck;
            } else {
                cur = out;
            }
        }
        if (failed) continue;
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            for (int j = 0; j < 3; ++j) {
                xT[3 * (b + i) + j] = cur.s.x[3 * i + j];
                vT[3 * (b + i) + j] = cur.s.v[3 * i + j];
                wT[3 * (b + i) + j] = cur.s.w[3 * i + j];
            }
            for (int j = 0; j < 4; ++j) qT[4 * (b + i) + j] = cur.s.q[4 * i + j];
        }
    }
}

__device__ void mapCacheAdjoint(const Slot &ws, const StepScratch<F> &prev, uint32_t count) {
    F *alam = at<F>(ws.base, ws.L.alam);
    const F *acache = at<F>(ws.base, ws.L.acache);
    for (uint32_t i = threadIdx.x; i < 12 * ws.maxM; i += blockDim.x) alam[i] = 0.0f;
    __syncthreads();
    for (uint32_t e = threadIdx.x; e < count; e += blockDim.x) {
        const uint32_t kp = prev.cacheSrc[e];
        for (int j = 0; j < 3; ++j) alam[3 * kp + j] += acache[3 * e + j];
    }
    __syncthreads();
}

// Adjoint: per segment (last first) recompute from the checkpoint with the
// tape, then reverse step by step.
__global__ void __launch_bounds__(128) k_rollout_backward(Args a, const F *gx, const F *gq, const F *gv,
                                                        const F *gw, F *gx0, F *gq0, F *gv0, F *gw0, F *gmass,
                                                        F *gmu, F *grest) {
    for (;;) {
        const uint32_t w = nextWorld(a);
        if (w >= a.worlds) return;
        const Slot ws = slotOf(a, w);
        unsigned char *base = ws.base;
        const Layout &L0 = ws.L;
        const WorldParams<F> W = params(a, w, ws);
        const uint32_t n = W.n, b = a.bodyStart[w];
        AdjointView<F> adj{at<F>(base, L0.ax),     at<F>(base, L0.aq),     at<F>(base, L0.av),
                           at<F>(base, L0.aw),     at<F>(base, L0.alam),   at<F>(base, L0.app),
                           at<F>(base, L0.apm),    at<F>(base, L0.an),     at<F>(base, L0.amuM),
                           at<F>(base, L0.arestM), at<F>(base, L0.acache), at<F>(base, L0.amass),
                           at<F>(base, L0.amu),    at<F>(base, L0.arest)};
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            for (int j = 0; j < 3; ++j) {
                adj.ax[3 * i + j] = gx ? gx[3 * (b + i) + j] : 0.0f;
                adj.av[3 * i + j] = gv ? gv[3 * (b + i) + j] : 0.0f;
                adj.aw[3 * i + j] = gw ? gw[3 * (b + i) + j] : 0.0f;
            }
            for (int j = 0; j < 4; ++j) adj.aq[4 * i + j] = gq ? gq[4 * (b + i) + j] : 0.0f;
            adj.amass[i] = adj.amu[i] = adj.arest[i] = 0.0f;
        }
        for (uint32_t i = threadIdx.x; i < 12 * ws.maxM; i += blockDim.x) adj.alam[i] = 0.0f;
        __syncthreads();
        ad::StateView<F> v1{nullptr, nullptr, at<F>(base, L0.v1v), at<F>(base, L0.v1w)};
        const uint32_t nSeg = (a.steps + a.ckEvery - 1) / a.ckEvery;
        bool pending = false, failed = false;
        uint32_t pendingCount = 0;
        for (int s = (int)nSeg - 1; s >= 0 && !failed; --s) {
            const uint32_t t0 = (uint32_t)s * a.ckEvery;
            const uint32_t L = min(a.steps, t0 + a.ckEvery) - t0;
            copySnap(snapshot(ws, (uint32_t)s, n), snapshot(ws, a.nCk, n), n);
            for (uint32_t i = 0; i < L; ++i) {
                const Snap in = snapshot(ws, a.nCk + i, n), out = snapshot(ws, a.nCk + i + 1, n);
                const StepScratch<F> sc = scratch(ws, i);
                forwardStep<F, BlockTeam>(W, in.s, in.c, out.s, out.c, sc, true);
                if (sc.counts[3]) {
                    if (threadIdx.x == 0) atomicOr(&a.err[w], sc.counts[3]);
                    failed = true;
                    break;
                }
            }
            if (failed) break;
            if (pending) mapCacheAdjoint(ws, scratch(ws, L - 1), pendingCount);
            for (int i = (int)L - 1; i >= 0; --i) {
                const Snap in = snapshot(ws, a.nCk + i, n), out = snapshot(ws, a.nCk + i + 1, n);
                const StepScratch<F> sc = scratch(ws, (uint32_t)i);
                backwardStep<F, BlockTeam>(W, in.s, in.c, out.s, v1, sc, adj);
                if (sc.counts[3]) {
                    if (threadIdx.x == 0) atomicOr(&a.err[w], sc.counts[3]);
                    failed = true;
                    break;
                }
                const uint32_t cnt = *in.c.count;
                if (i > 0) {
                    mapCacheAdjoint(ws, scratch(ws, (uint32_t)i - 1), cnt);
                } else {
                    pending = t0 > 0;
                    pendingCount = cnt;
                }
            }
        }
        if (failed) continue;
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            for (int j = 0; j < 3; ++j) {
                if (gx0) gx0[3 * (b + i) + j] = adj.ax[3 * i + j];
                if (gv0) gv0[3 * (b + i) + j] = adj.av[3 * i + j];
                if (gw0) gw0[3 * (b + i) + j] = adj.aw[3 * i + j];
            }
            for (int j = 0; j < 4; ++j)
                if (gq0) gq0[4 * (b + i) + j] = adj.aq[4 * i + j];
            if (gmass) gmass[b + i] = adj.amass[i];
            if (gmu) gmu[b + i] = adj.amu[i];
            if (grest) grest[b + i] = adj.arest[i];
        }
    }
}

template <class T> void uploadVec(DeviceArray<T> &d, const std::vector<T> &h) {
    d.reserve(h.size());
    if (!h.empty()) PE_CHECK(cudaMemcpy(d.ptr, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
}

} // namespace

Rollout::Rollout(int device) : device_(device) {
    PE_CHECK(cudaSetDevice(device_));
    PE_CHECK(cudaEventCreate(&e0_));
    PE_CHECK(cudaEventCreate(&e1_));
    PE_CHECK(cudaMallocHost(&hostErr_, sizeof(uint32_t)));
}

Rollout::~Rollout() {
    if (e0_) cudaEventDestroy(e0_);
    if (e1_) cudaEventDestroy(e1_);
    if (hostErr_) cudaFreeHost(hostErr_);
}

void Rollout::create(const std::vector<uint32_t> &worldBodies, const std::vector<uint8_t> &shape,
                     const std::vector<uint8_t> &isStatic, const std::vector<float> &halfExtents,
                     const std::vector<float> &invInertia, uint32_t steps, float dt, int iterations,
                     uint32_t checkpointEvery) {
    PE_CHECK(cudaSetDevice(device_));
    if (worldBodies.empty()) throw std::invalid_argument("a rollout needs at least one world");
    if (steps == 0) throw std::invalid_argument("a rollout needs at least one step");
    if (checkpointEvery == 0) throw std::invalid_argument("checkpoint interval must be positive");
    if (iterations < 0 || iterations > 256) throw std::invalid_argument("iterations out of range");
    uint64_t total = 0;
    nMax_ = 0;
    std::vector<uint32_t> start(worldBodies.size() + 1, 0);
    for (size_t w = 0; w < worldBodies.size(); ++w) {
        if (worldBodies[w] == 0 || worldBodies[w] > kRolloutMaxBodies)
            throw std::invalid_argument("a differentiable world holds 1 to " + std::to_string(kRolloutMaxBodies) +
                                        " bodies");
        start[w] = (uint32_t)total;
        total += worldBodies[w];
        nMax_ = std::max(nMax_, worldBodies[w]);
    }
    start.back() = (uint32_t)total;
    if (shape.size() != total || isStatic.size() != total || halfExtents.size() != 3 * total ||
        invInertia.size() != 3 * total)
        throw std::invalid_argument("per-body arrays must hold the sum of the world body counts");
    for (uint8_t s : shape)
        if (s > 1) throw std::invalid_argument("differentiable worlds hold spheres and boxes");
    nb_ = total;
    worldBodies_ = worldBodies;
    steps_ = steps;
    dt_ = dt;
    iterations_ = iterations;
    ckEvery_ = std::min(checkpointEvery, steps);
    nCk_ = (steps + ckEvery_ - 1) / ckEvery_ + 1;
    // worlds are taken largest first
    std::vector<uint32_t> order(worldBodies.size());
    for (size_t w = 0; w < order.size(); ++w) order[w] = (uint32_t)w;
    std::stable_sort(order.begin(), order.end(),
                     [&](uint32_t x, uint32_t y) { return worldBodies[x] > worldBodies[y]; });
    uploadVec(order_, order);
    uploadVec(bodyStart_, start);
    uploadVec(shape_, shape);
    uploadVec(static_, isStatic);
    uploadVec(dims_, halfExtents);
    uploadVec(iinv_, invInertia);
    mass_.reserve(total);
    mu_.reserve(total);
    rest_.reserve(total);
    queue_.reserve(1);
    err_.reserve(worldBodies.size());
    arena_.release();
    haveForward_ = false;
}

void Rollout::setManifoldCapacity(float perBody) {
    if (!(perBody >= 0.25f && perBody <= 64.0f))
        throw std::invalid_argument("manifold capacity must be 0.25 to 64 manifolds per body");
    const uint32_t q = (uint32_t)(perBody * 4.0f + 0.5f);
    if (q == quarterPerBody_) return;
    quarterPerBody_ = q;
    arena_.release();  // laid out again at the next forward call
    haveForward_ = false;
}

// Every world's slot is sized by its own body count (checkpoints, one
// segment's step scratch and tape, adjoints), allocated at the first forward
// call after creation or a capacity change.
void Rollout::ensureArena() {
    if (arena_.ptr) return;
    std::vector<unsigned long long> off(worldBodies_.size());
    unsigned long long arenaBytes = 0;
    for (size_t w = 0; w < worldBodies_.size(); ++w) {
        const uint32_t n = worldBodies_[w];
        const Layout L = makeLayout(n, worldMaxPairs(n), worldMaxManifolds(n, quarterPerBody_), iterations_,
                                    nCk_ + ckEvery_ + 1, ckEvery_);
        off[w] = arenaBytes;
        arenaBytes += align16(L.stride);
    }
    uploadVec(worldOff_, off);
    arena_.reserve(arenaBytes);
    bytes_ = arenaBytes + nb_ * 64;
}

void Rollout::checkErrors(cudaStream_t s, const char *what) {
    std::vector<uint32_t> e(worldBodies_.size());
    PE_CHECK(cudaMemcpyAsync(e.data(), err_.ptr, e.size() * 4, cudaMemcpyDeviceToHost, s));
    PE_CHECK(cudaStreamSynchronize(s));
    for (size_t w = 0; w < e.size(); ++w)
        if (e[w]) {
            const uint32_t b = e[w];
            const char *m = (b & kAdErrPairs)       ? "candidate pairs exceed the world's capacity"
                            : (b & kAdErrManifolds) ? "contact manifolds exceed the world's capacity"
                            : (b & kAdErrColors)    ? "solver colouring failed"
                            : (b & kAdErrCache)     ? "warm-start cache overflow"
                                                    : "the adjoint's replay of a contact differed from the forward";
            throw std::runtime_error(std::string(what) + ": world " + std::to_string(w) + ": " + m);
        }
}

void Rollout::forward(const float *x0, const float *q0, const float *v0, const float *w0, const float *mass,
                      const float *friction, const float *restitution, float *xT, float *qT, float *vT, float *wT,
                      cudaStream_t s) {
    PE_CHECK(cudaSetDevice(device_));
    if (!x0 || !q0 || !v0 || !w0 || !mass || !friction || !restitution || !xT || !qT || !vT || !wT)
        throw std::invalid_argument("null argument");
    ensureArena();
    PE_CHECK(cudaMemcpyAsync(mass_.ptr, mass, nb_ * 4, cudaMemcpyDeviceToDevice, s));
    PE_CHECK(cudaMemcpyAsync(mu_.ptr, friction, nb_ * 4, cudaMemcpyDeviceToDevice, s));
    PE_CHECK(cudaMemcpyAsync(rest_.ptr, restitution, nb_ * 4, cudaMemcpyDeviceToDevice, s));
    PE_CHECK(cudaMemsetAsync(queue_.ptr, 0, 4, s));
    PE_CHECK(cudaMemsetAsync(err_.ptr, 0, worldBodies_.size() * 4, s));
    Args a{};
    a.arena = arena_.ptr;
    a.quarterPerBody = quarterPerBody_;
    a.worldOff = worldOff_.ptr;
    a.order = order_.ptr;
    a.bodyStart = bodyStart_.ptr;
    a.shape = shape_.ptr;
    a.isStatic = static_.ptr;
    a.dims = dims_.ptr;
    a.iinv = iinv_.ptr;
    a.mass = mass_.ptr;
    a.mu = mu_.ptr;
    a.rest = rest_.ptr;
    a.worlds = (uint32_t)worldBodies_.size();
    a.steps = steps_;
    a.ckEvery = ckEvery_;
    a.nCk = nCk_;
    a.iterations = iterations_;
    a.gx = gravity[0];
    a.gy = gravity[1];
    a.gz = gravity[2];
    a.dt = dt_;
    a.queueHead = queue_.ptr;
    a.err = err_.ptr;
    int sms = 0;
    PE_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
    int per = 0;
    PE_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_rollout_forward, 128, 0));
    const uint32_t blocks = std::min<uint32_t>(a.worlds, (uint32_t)std::max(1, per) * sms);
    PE_CHECK(cudaEventRecord(e0_, s));
    k_rollout_forward<<<blocks, 128, 0, s>>>(a, x0, q0, v0, w0, xT, qT, vT, wT);
    PE_LAUNCHED();
    PE_CHECK(cudaEventRecord(e1_, s));
    checkErrors(s, "rollout forward");
    float ms = 0;
    PE_CHECK(cudaEventElapsedTime(&ms, e0_, e1_));
    fwdMs_ = ms;
    haveForward_ = true;
}

void Rollout::backward(const float *gx, const float *gq, const float *gv, const float *gw, float *gx0, float *gq0,
                       float *gv0, float *gw0, float *gmass, float *gfriction, float *grestitution, cudaStream_t s) {
    PE_CHECK(cudaSetDevice(device_));
    if (!haveForward_) throw std::invalid_argument("backward needs a forward call first");
    PE_CHECK(cudaMemsetAsync(queue_.ptr, 0, 4, s));
    PE_CHECK(cudaMemsetAsync(err_.ptr, 0, worldBodies_.size() * 4, s));
    Args a{};
    a.arena = arena_.ptr;
    a.quarterPerBody = quarterPerBody_;
    a.worldOff = worldOff_.ptr;
    a.order = order_.ptr;
    a.bodyStart = bodyStart_.ptr;
    a.shape = shape_.ptr;
    a.isStatic = static_.ptr;
    a.dims = dims_.ptr;
    a.iinv = iinv_.ptr;
    a.mass = mass_.ptr;
    a.mu = mu_.ptr;
    a.rest = rest_.ptr;
    a.worlds = (uint32_t)worldBodies_.size();
    a.steps = steps_;
    a.ckEvery = ckEvery_;
    a.nCk = nCk_;
    a.iterations = iterations_;
    a.gx = gravity[0];
    a.gy = gravity[1];
    a.gz = gravity[2];
    a.dt = dt_;
    a.queueHead = queue_.ptr;
    a.err = err_.ptr;
    int sms = 0;
    PE_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
    int per = 0;
    PE_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_rollout_backward, 128, 0));
    const uint32_t blocks = std::min<uint32_t>(a.worlds, (uint32_t)std::max(1, per) * sms);
    PE_CHECK(cudaEventRecord(e0_, s));
    k_rollout_backward<<<blocks, 128, 0, s>>>(a, gx, gq, gv, gw, gx0, gq0, gv0, gw0, gmass, gfriction,
                                              grestitution);
    PE_LAUNCHED();
    PE_CHECK(cudaEventRecord(e1_, s));
    checkErrors(s, "rollout backward");
    float ms = 0;
    PE_CHECK(cudaEventElapsedTime(&ms, e0_, e1_));
    bwdMs_ = ms;
}

} // namespace pe
