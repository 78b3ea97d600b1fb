// Sleeping islands on the device (PhysicsWorld sleeping,
// src/world/physics_world.cpp:341-516, and the solver's sleeping rules,
// src/solver/sequential_impulse_solver.cpp:317-324, :623-646).
//
//   k_sleep_contacts : wakeSleepIslands' contact loop (:393-409): union of the
//                      dynamic bodies of every contact, and a static body with a
//                      wake request wakes its dynamic partner.
//   k_sleep_islands  : per-island OR of awake / sleeping / wake-request (:410-419).
//   k_sleep_apply    : islands with a wake request, or with awake and sleeping
//                      bodies, wake (:420-431); inside a step also the gravity
//                      integration of bodies the contacts woke (:741-748) and the
//                      solver's per-body sleeping bit.
//   k_sleep_finish   : finishSleeping's sleep decision (:494-515) after the pose
//                      kernel folded each body's quiet time into its island.
//   k_cache_carry_*  : warm-start entries of contacts among sleeping and static
//                      bodies carried into the next cache (:626-646), merged
//                      with the solver's entries in key order.
//
// Islands are found with a lock-free union-find whose roots are the smallest
// body index of each island (a larger root is always hooked under a smaller
// one), which is the partition the reference's sleepRoot builds; everything an
// island aggregates (OR of flags, minimum quiet time) is independent of the
// order in which contacts join it.
#include "pe_bodies.cuh"
#include "pe_kernels.cuh"
#include "pe_prims.cuh"
#include "pe_stages.h"

namespace pe {

namespace {

constexpr uint32_t kIslandAwake = 1u, kIslandSleeping = 2u, kIslandWake = 4u;
constexpr int kSleepThreads = 256;

// Root of body i (bounded walk; parents only ever move to smaller indices).
__device__ __forceinline__ uint32_t sleepFind(const uint32_t *parent, uint32_t i, uint32_t nb) {
    for (uint32_t n = 0; n <= nb; ++n) {
        const uint32_t p = ldvol(&parent[i]);
        if (p == i) return i;
        i = p;
    }
    return i;
}

__device__ __forceinline__ void sleepUnite(uint32_t *parent, uint32_t a, uint32_t b, uint32_t nb, uint32_t *err) {
    for (uint32_t spins = 0; spins < spinLimit(); ++spins) {
        a = sleepFind(parent, a, nb);
        b = sleepFind(parent, b, nb);
        if (a == b) return;
        const uint32_t hi = a > b ? a : b, lo = a > b ? b : a;
        const uint32_t old = atomicCAS(&parent[hi], hi, lo);
        if (old == hi) return;
        a = old;  // hi was hooked meanwhile: continue from its new parent
        b = lo;
    }
    atomicOr(err, kErrTimeout);
}

// RigidBody::wakeUp on a dynamic body.
__device__ __forceinline__ void wakeBody(uint32_t *flags, uint32_t i) {
    atomicAnd(&flags[i], ~kSleepAsleep);
    atomicOr(&flags[i], kSleepWake);
}

__device__ __forceinline__ bool bodyLive(const WorldView &w, uint32_t i, uint32_t gen) {
    return i < w.nb && (w.bflags[i] & kBodyAlive) && w.bgen[i] == gen;
}

inline uint32_t gridFor(uint32_t n) {
    const uint32_t b = (n + kSleepThreads - 1) / kSleepThreads;
    return b ? (b < 1024u ? b : 1024u) : 1u;
}

} // namespace

// Per-body reset of the island scratch (parent = self, no island flags).
__global__ void k_sleep_reset(WorldView w) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < w.nb; i += gridDim.x * blockDim.x) {
        w.sleepParent[i] = i;
        w.sleepIsland[i] = 0u;
    }
}

// Contacts m < M (M from d_M when given, else Mhost).  flags: the sleep flags
// being updated (the world's committed copy before a step, the step's output
// copy inside it).
__global__ void k_sleep_contacts(WorldView w, ManifoldView mv, const uint32_t *d_M, uint32_t Mhost, uint32_t mcap,
                                 uint32_t *flags, uint32_t *err) {
    uint32_t M = d_M ? *d_M : Mhost;
    M = M < mcap ? M : mcap;
    for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
        const uint32_t ia = mv.bodyA[m], ib = mv.bodyB[m];
        if (!bodyLive(w, ia, mv.genA[m]) || !bodyLive(w, ib, mv.genB[m]) || mv.pointCount[m] == 0) continue;
        const bool sa = (w.bflags[ia] & kBodyStatic) != 0, sb = (w.bflags[ib] & kBodyStatic) != 0;
        if (!sa && !sb) {
            sleepUnite(w.sleepParent, ia, ib, w.nb, err);
        } else if (sa && (flags[ia] & kSleepWake) && !sb) {
            wakeBody(flags, ib);
        } else if (sb && (flags[ib] & kSleepWake) && !sa) {
            wakeBody(flags, ia);
        }
    }
}

// Per live dynamic body: island root (stored as its parent) and the island's
// awake / sleeping / wake-request bits.
__global__ void k_sleep_islands(WorldView w, const uint32_t *flags) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < w.nb; i += gridDim.x * blockDim.x) {
        const uint32_t bf = w.bflags[i];
        if (!(bf & kBodyAlive) || (bf & kBodyStatic)) continue;
        const uint32_t r = sleepFind(w.sleepParent, i, w.nb);
        const uint32_t f = flags[i];
        const uint32_t bits = ((f & kSleepAsleep) ? kIslandSleeping : kIslandAwake) | ((f & kSleepWake) ? kIslandWake : 0u);
        if ((ldvol(&w.sleepIsland[r]) & bits) != bits) atomicOr(&w.sleepIsland[r], bits);
    }
}

// Per live dynamic body: wake the islands that must wake.  inStep: the body
// state is the step's output copy; bodies woken after the gravity pass get
// their gravity now, and bflags receives the solver's sleeping bit.
__global__ void k_sleep_apply(WorldView w, uint32_t *flags, float *quiet, uint32_t *bflags, int inStep, DevStats *st) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < w.nb; i += gridDim.x * blockDim.x) {
        const uint32_t bf = w.bflags[i];
        if (!(bf & kBodyAlive) || (bf & kBodyStatic)) {
            if (inStep) bflags[i] = bf & ~kBodySleeping;
            continue;
        }
        uint32_t f = flags[i];
        const uint32_t r = sleepFind(w.sleepParent, i, w.nb);
        const uint32_t isl = w.sleepIsland[r];
        if ((isl & kIslandWake) || ((isl & kIslandAwake) && (isl & kIslandSleeping))) {
            f = (f & ~kSleepAsleep) | kSleepWake;
            quiet[i] = 0.0f;
        }
        if (inStep) {
            if (!(f & kSleepIntegrated) && !(f & kSleepAsleep)) {
                const V3 force = w.force ? f4xyz(w.force[i]) : V3{0.0f, 0.0f, 0.0f};
                const V3 lin = integrateVelocity(f4xyz(w.nxt.lin[i]), V3{w.gx, w.gy, w.gz}, force, w.mat[i].x, w.dt);
                w.nxt.lin[i] = make4(lin, 0.0f);
                f |= kSleepIntegrated;
            }
            w.sleepParent[i] = r;  // flattened for the pose and finish kernels
            bflags[i] = (f & kSleepAsleep) ? (bf | kBodySleeping) : (bf & ~kBodySleeping);
            if (!(f & kSleepAsleep)) aggregatedAdd32(&st->awakeInStep, 1u);
        }
        flags[i] = f;
    }
}

// finishSleeping's second loop: islands whose least quiet time reached the
// limit sleep with zero velocities; wake requests are cleared; the live
// dynamic bodies are counted awake / asleep.  The last block copies the step's
// counters to the pinned host mirror (hostOut, nullable).
__global__ void k_sleep_finish(WorldView w, DevStats *st, DevStats *hostOut, uint32_t *done) {
    const float timeToSleep = 0.5f;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t awake = 0, asleep = 0;
    if (i < w.nb) {
        const uint32_t bf = w.bflags[i];
        if (bf & kBodyAlive) {
            uint32_t f = w.sleepOut[i];
            if (!(bf & kBodyStatic)) {
                const float islandQuiet = __uint_as_float(w.sleepQuietMin[w.sleepParent[i]]);
                if (islandQuiet >= timeToSleep) {
                    f |= kSleepAsleep;
                    w.nxt.lin[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    w.nxt.ang[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                }
                if (f & kSleepAsleep) asleep = 1;
                else awake = 1;
            }
            w.sleepOut[i] = f & ~(kSleepWake | kSleepIntegrated);
        }
    }
    if (awake) aggregatedAdd32(&st->awakeBodies, 1u);
    if (asleep) aggregatedAdd32(&st->sleepingBodies, 1u);
    if (!hostOut) return;
    __syncthreads();
    __shared__ bool s_last;
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        const unsigned long long *src = reinterpret_cast<const unsigned long long *>(st);
        unsigned long long *dst = reinterpret_cast<unsigned long long *>(hostOut);
        for (uint32_t k = threadIdx.x; k < sizeof(DevStats) / 8; k += blockDim.x) dst[k] = __ldcg(&src[k]);
        if (threadIdx.x == 0) *done = 0;
    }
}

// Carry flags of the old warm-start cache: both bodies live with the entry's
// generations, at least one asleep, neither moving (sequential_impulse_solver.cpp:633-643).
__global__ void k_cache_carry_flags(WorldView w, CacheView oc, const uint32_t *oldCount, uint32_t cap,
                                    uint32_t *carry) {
    uint32_t n = *oldCount;
    n = n < cap ? n : cap;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const unsigned long long k = oc.key[e], g = oc.gens[e];
        const uint32_t ia = (uint32_t)(k >> 32), ib = (uint32_t)k;
        bool c = false;
        if (bodyLive(w, ia, (uint32_t)(g >> 32)) && bodyLive(w, ib, (uint32_t)g)) {
            const uint32_t fa = w.bflags[ia], fb = w.bflags[ib];
            const bool sleepA = (fa & kBodySleeping) != 0, sleepB = (fb & kBodySleeping) != 0;
            c = (sleepA || sleepB) && (sleepA || (fa & kBodyStatic)) && (sleepB || (fb & kBodyStatic));
        }
        carry[e] = c ? 1u : 0u;
    }
}

namespace {
// First index in keys[0, n) whose key is not less than k.
__device__ __forceinline__ uint32_t lowerBoundKey(const unsigned long long *keys, uint32_t n, unsigned long long k) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (keys[mid] < k) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}
__device__ __forceinline__ void copyEntry(const CacheView &from, uint32_t i, const CacheView &to, uint32_t j) {
    to.key[j] = from.key[i];
    to.gens[j] = from.gens[i];
    to.anchorA[j] = from.anchorA[i];
    to.anchorB[j] = from.anchorB[i];
    to.tangent2[j] = from.tangent2[i];
}
} // namespace

// Next cache = carried old entries + the solver's entries (tc, sorted), merged
// in key order (the two key sets are disjoint: a carried pair is not solved).
// carryPos: exclusive scan of the carry flags, carryTotal its sum.
__global__ void k_cache_merge(CacheView oc, const uint32_t *oldCount, const uint32_t *carry, const uint32_t *carryPos,
                              const uint32_t *carryTotal, CacheView tc, const uint32_t *tmpCount, CacheView nc,
                              uint32_t *newCount, uint32_t cap, DevStats *st) {
    uint32_t no = *oldCount, nt = *tmpCount;
    no = no < cap ? no : cap;
    nt = nt < cap ? nt : cap;
    const uint32_t total = *carryTotal;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    if (tid == 0) {
        const uint32_t n = total + nt;
        *newCount = n < cap ? n : cap;
        st->carried = total;
        if (n > cap) atomicOr(&st->err, kErrCacheCapacity);
    }
    for (uint32_t e = tid; e < no; e += stride) {
        if (!carry[e]) continue;
        const uint32_t at = carryPos[e] + lowerBoundKey(tc.key, nt, oc.key[e]);
        if (at < cap) copyEntry(oc, e, nc, at);
    }
    for (uint32_t j = tid; j < nt; j += stride) {
        const uint32_t lb = lowerBoundKey(oc.key, no, tc.key[j]);
        const uint32_t at = j + (lb < no ? carryPos[lb] : total);
        if (at < cap) copyEntry(tc, j, nc, at);
    }
}

// The solver's sleeping bit of every body from committed sleep flags.
__global__ void k_sleep_bits(WorldView w, const uint32_t *flags, uint32_t *bflags, DevStats *st) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < w.nb; i += gridDim.x * blockDim.x) {
        const uint32_t bf = w.bflags[i];
        const bool dyn = (bf & kBodyAlive) && !(bf & kBodyStatic);
        const bool asleep = dyn && (flags[i] & kSleepAsleep);
        bflags[i] = asleep ? (bf | kBodySleeping) : (bf & ~kBodySleeping);
        if (dyn && !asleep) aggregatedAdd32(&st->awakeInStep, 1u);
    }
}

// ------------------------------------------------------------- launchers ---
void launchSleepBits(const WorldView &w, const uint32_t *flags, uint32_t *bflags, DevStats *st, cudaStream_t s) {
    if (!w.nb) return;
    k_sleep_bits<<<gridFor(w.nb), kSleepThreads, 0, s>>>(w, flags, bflags, st);
    PE_LAUNCHED();
}

void launchSleepWake(const WorldView &w, const ManifoldView &mv, uint32_t Mhost, uint32_t mcap, uint32_t *flags,
                     float *quiet, uint32_t *err, cudaStream_t s) {
    if (!w.nb) return;
    k_sleep_reset<<<gridFor(w.nb), kSleepThreads, 0, s>>>(w);
    PE_LAUNCHED();
    if (Mhost) {
        k_sleep_contacts<<<gridFor(Mhost), kSleepThreads, 0, s>>>(w, mv, nullptr, Mhost, mcap, flags, err);
        PE_LAUNCHED();
    }
    k_sleep_islands<<<gridFor(w.nb), kSleepThreads, 0, s>>>(w, flags);
    PE_LAUNCHED();
    k_sleep_apply<<<gridFor(w.nb), kSleepThreads, 0, s>>>(w, flags, quiet, nullptr, 0, nullptr);
    PE_LAUNCHED();
}

void launchSleepContacts(const WorldView &w, const ManifoldView &mv, DevStats *st, uint32_t mcap, uint32_t *bflags,
                         cudaStream_t s) {
    if (!w.nb) return;
    const uint32_t span = 4u * (uint32_t)smCount() * kSleepThreads;
    k_sleep_contacts<<<gridFor(mcap < span ? mcap : span), kSleepThreads, 0, s>>>(w, mv, &st->manifolds, 0u, mcap, w.sleepOut, &st->err);
    PE_LAUNCHED();
    k_sleep_islands<<<gridFor(w.nb), kSleepThreads, 0, s>>>(w, w.sleepOut);
    PE_LAUNCHED();
    k_sleep_apply<<<gridFor(w.nb), kSleepThreads, 0, s>>>(w, w.sleepOut, w.quietOut, bflags, 1, st);
    PE_LAUNCHED();
}

void launchSleepFinish(const WorldView &w, DevStats *st, DevStats *hostOut, uint32_t *done, cudaStream_t s) {
    if (!w.nb) return;
    k_sleep_finish<<<(w.nb + kSleepThreads - 1) / kSleepThreads, kSleepThreads, 0, s>>>(w, st, hostOut, done);
    PE_LAUNCHED();
}

void launchCacheCarry(const WorldView &w, const CacheView &oldCache, const uint32_t *oldCount, const CacheView &tmp,
                      const uint32_t *tmpCount, const CacheView &newCache, uint32_t *newCount, uint32_t cap,
                      uint32_t *carry, uint32_t *carryPos, uint32_t *carryTotal, DevStats *st, Scratch &ws,
                      cudaStream_t s) {
    const uint32_t span = 4u * (uint32_t)smCount() * kSleepThreads;
    const uint32_t g = gridFor(cap < span ? cap : span);
    k_cache_carry_flags<<<g, kSleepThreads, 0, s>>>(w, oldCache, oldCount, cap, carry);
    PE_LAUNCHED();
    launchScanExclusive(carry, carryPos, oldCount, cap, carryTotal, ws, &st->err, s);
    k_cache_merge<<<g, kSleepThreads, 0, s>>>(oldCache, oldCount, carry, carryPos, carryTotal, tmp, tmpCount, newCache,
                                              newCount, cap, st);
    PE_LAUNCHED();
}

void setSpinLimitSleep(uint32_t limit) { setSpinLimitOfUnit(limit); }

} // namespace pe
