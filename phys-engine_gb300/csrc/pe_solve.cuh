// Solver pieces shared by the single-world pipeline and the batched-world kernel.
#pragma once
#include "pe_block.cuh"
#include "pe_kernels.cuh"
#include "pe_engine.h"
#include "pe_stages.h"

namespace pe {

constexpr uint32_t kUncolored = 0xFFFFFFFFu;
// Colour windows.  The per-body masks of the Jones-Plassmann colouring hold
// kMaxColors colours: the window [base, base + kMaxColors).  A manifold whose
// higher-priority neighbours already use every colour of the window is
// deferred (kDeferred): its greedy colour lies above the window and depends
// only on the colours of its deferred higher-priority neighbours, so the
// deferred manifolds are coloured again, by the same rule, in the next window
// (masks cleared, colours offset by kMaxColors).  There is no colour limit.
constexpr uint32_t kDeferred = 0xFFFFFFFEu;
// Rounds of one colour window (a window takes at least as many rounds as the
// largest number of its manifolds at one body).
constexpr uint32_t kMaxRounds = 4096;
constexpr int kSolveThreads = 256;
constexpr int kBlockSolveThreads = 512;

__device__ __forceinline__ uint32_t colorPriority(uint32_t m) {
    uint32_t h = m;
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

__device__ __forceinline__ float4 ld4(const float4 *p) { return __ldcg(p); }
__device__ __forceinline__ void st4(float4 *p, const float4 &v) { __stcg(p, v); }


struct SolveArgs {
    WorldView w;
    ManifoldView mv;
    SolverBuffers sb;
    CacheView oldCache;
    const uint32_t *oldCount;
    DevStats *st;
    uint32_t mcap;
    int iterations;
    // Collider i belongs to body i for every live collider: manifold (pair)
    // order is then (body A, body B) order with one manifold per key, which is
    // already the order of the rebuilt warm-start cache.
    bool pairOrderCache;
    // Manifolds the solver takes, [0, *count): the step's manifold count, or
    // with sleeping on zero when no body is awake (every contact is skipped).
    const uint32_t *count;
};

// Where the velocity iterations read and write body velocities: the world's
// arrays by body index, or shared-memory copies by staging slot.
struct GlobalVel {
    const SolveArgs &a;
    __device__ __forceinline__ uint2 bodies(uint32_t, uint32_t m) const { return a.sb.pbody[m]; }
    __device__ __forceinline__ V3 lin(uint32_t b) const { return f4xyz(ld4(&a.w.nxt.lin[b])); }
    __device__ __forceinline__ V3 ang(uint32_t b) const { return f4xyz(ld4(&a.w.nxt.ang[b])); }
    __device__ __forceinline__ void store(uint32_t b, const V3 &l, const V3 &w) const {
        st4(&a.w.nxt.lin[b], make4(l, 0.0f));
        st4(&a.w.nxt.ang[b], make4(w, 0.0f));
    }
};
struct SharedVel {
    float4 *v;          // slot s: lin at 2s, ang at 2s + 1
    const uint2 *slot;  // per solve index k: slots of body A and body B
    __device__ __forceinline__ uint2 bodies(uint32_t k, uint32_t) const { return slot[k]; }
    __device__ __forceinline__ V3 lin(uint32_t s) const { return f4xyz(v[2 * s]); }
    __device__ __forceinline__ V3 ang(uint32_t s) const { return f4xyz(v[2 * s + 1]); }
    __device__ __forceinline__ void store(uint32_t s, const V3 &l, const V3 &w) const {
        v[2 * s] = make4(l, 0.0f);
        v[2 * s + 1] = make4(w, 0.0f);
    }
};

struct BlockSolveShared {
    uint32_t start[kMaxColors + 1];
    uint32_t count[kMaxColors];
    uint32_t scan[40];
    uint32_t colored;
    uint32_t colors;
    uint32_t slots;
    uint32_t deferred;  // manifolds deferred to the next colour window
};

// Solve-index range [first, end) of colour c: from the shared ranges, or
// from sb.colorStart when the step has more than kMaxColors colours.
__device__ __forceinline__ uint2 colorRange(const BlockSolveShared &sh, const SolverBuffers &sb, uint32_t c,
                                            uint32_t C, uint32_t M) {
    if (C <= (uint32_t)kMaxColors) return make_uint2(sh.start[c], sh.start[c + 1]);
    return make_uint2(__ldcg(&sb.colorStart[c]), c + 1 < C ? __ldcg(&sb.colorStart[c + 1]) : M);
}

// Shared-memory copies of the velocities of the bodies the manifolds touch,
// used by the single-block solver for the warm start and the iterations.
struct VelStage {
    float4 *v;            // [2 * cap]
    uint2 *slot;          // [maxM] slots of body A / body B per solve index
    uint32_t *slotBody;   // [cap] body of each slot
    uint32_t cap;
};
constexpr uint32_t kSlotFree = 0xFFFFFFFFu;

// With sleeping on, a manifold among static and sleeping bodies only is not
// solved, cached or counted (sequential_impulse_solver.cpp:321-324).
__device__ __forceinline__ bool solvedPair(const WorldView &w, uint32_t flA, uint32_t flB) {
    return !w.sleepMode || bodyMoves(flA) || bodyMoves(flB);
}

// --------------------------------------------------------------- prepare ---
// prepareBody (:275-287) + prepareContactPoints (:101-214) + the cache lookup
// of warmStartPrepared (:448-490).  Data are written by manifold index m (no
// dependence on the solve order, so prepare may run before the colouring).
// Work items are (manifold, point) pairs q = p M + m (all point-0 items first,
// so consecutive threads take consecutive manifolds): a manifold's points are
// independent here, so the slowest point, not the sum of a manifold's points,
// bounds the pass.  Each item reads its manifold's data; point 0's item also
// writes the per-manifold outputs.

// One item's manifold data.  Every field is requested at once (the point's
// anchors and impulse are in bounds for any p < 4), before the item is known
// to be live.
struct PrepItem {
    uint32_t m, p, npts, ia, ib, gA, gB;
    float4 nf, aa, ab, imp;
    float rest;
};
__device__ __forceinline__ PrepItem loadPrepItemAt(const SolveArgs &a, uint32_t m, uint32_t p) {
    PrepItem t;
    t.m = m;
    t.p = p;
    t.npts = a.mv.pointCount[m];
    t.ia = a.mv.bodyA[m];
    t.ib = a.mv.bodyB[m];
    t.gA = a.mv.genA[m];
    t.gB = a.mv.genB[m];
    t.nf = a.mv.normalFriction[m];
    t.rest = a.mv.restitution[m];
    t.aa = a.mv.anchorA[4 * m + p];
    t.ab = a.mv.anchorB[4 * m + p];
    t.imp = a.mv.impulse[4 * m + p];
    return t;
}
__device__ __forceinline__ PrepItem loadPrepItem(const SolveArgs &a, uint32_t q, uint32_t M) {
    const uint32_t p = q / M;
    return loadPrepItemAt(a, q - p * M, p);
}

struct PrepTally {
    uint64_t prepared = 0, comparisons = 0, matches = 0;
    uint32_t solved = 0;
};
__device__ __forceinline__ void flushPrepTally(const SolveArgs &a, const PrepTally &t) {
    aggregatedAdd32(&a.st->solved, t.solved);
    aggregatedAdd64(&a.st->preparedPoints, t.prepared);
    aggregatedAdd64(&a.st->warmComparisons, t.comparisons);
    aggregatedAdd64(&a.st->warmMatches, t.matches);
}

// Prepares one item.  The bodies' data are requested first (indices clamped to
// a live entry); the cache range is searched while they are on their way, and
// the range's first four entries are requested before the body data are used,
// so an item costs two dependent memory round trips after its manifold data.
// cacheKeys: the old cache's keys (a shared-memory copy when they fit; the
// global array otherwise), cacheN of them.
// Cache entries [rb, re) of the body pair (ia, ib) in the sorted cache keys:
// the reference's equal_range (sequential_impulse_solver.cpp:448-456).
__device__ __forceinline__ uint2 cacheRange(const unsigned long long *cacheKeys, uint32_t cacheN, uint32_t ia,
                                            uint32_t ib) {
    const unsigned long long key = ((unsigned long long)ia << 32) | ib;
    uint32_t lo = 0, hi = cacheN;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (cacheKeys[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    uint32_t re = lo;
    while (re < cacheN && cacheKeys[re] == key) ++re;
    return make_uint2(lo, re);
}

// cacheRange for a cache larger than shared memory holds: `sample` holds every
// stride-th key (sample[i] = key[i stride], nS entries, stride <= kCacheSampleStride)
// in shared memory; the search there leaves a window of stride keys that holds the
// range's start, which is read from memory in one round trip with the entries
// after it.  Same result as cacheRange on the whole array.
constexpr uint32_t kCacheSampleStride = 8;
__device__ __forceinline__ uint2 cacheRangeSampled(const unsigned long long *sample, uint32_t nS, uint32_t stride,
                                                   const unsigned long long *cacheKeys, uint32_t cacheN,
                                                   uint32_t ia, uint32_t ib) {
    const unsigned long long key = ((unsigned long long)ia << 32) | ib;
    uint32_t lo = 0, hi = nS;  // first sample >= key
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (sample[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    // the first key >= key lies in [base, base + stride)
    const uint32_t base = lo ? (lo - 1) * stride + 1 : 0u;
    constexpr uint32_t W = kCacheSampleStride + 4;
    unsigned long long v[W];
#pragma unroll
    for (uint32_t j = 0; j < W; ++j) v[j] = base + j < cacheN ? __ldcg(&cacheKeys[base + j]) : ~0ull;
    uint32_t rb = base, re = base;
#pragma unroll
    for (uint32_t j = 0; j < W; ++j) {
        rb += (base + j < cacheN && v[j] < key) ? 1u : 0u;
        re += (base + j < cacheN && v[j] <= key) ? 1u : 0u;
    }
    // a run of equal keys longer than the window continues in memory
    while (re < cacheN && re == base + W && __ldcg(&cacheKeys[re]) == key) ++re;
    return make_uint2(rb, re);
}

__device__ __forceinline__ void prepareItem(const SolveArgs &a, const PrepItem &t,
                                            const unsigned long long *cacheKeys, uint32_t cacheN, PrepTally &tally,
                                            const uint2 *range = nullptr) {
    const uint32_t mcap = a.mcap;
    const WorldView &w = a.w;
    const uint32_t m = t.m, p = t.p, k = m;  // k: data index
    const uint32_t live = t.npts < 4u ? t.npts : 4u;  // live points (at most four)
    if (p > 0 && p >= live) return;
    const uint32_t ia = t.ia, ib = t.ib;
    const uint32_t ca = ia < w.nb ? ia : 0u, cb = ib < w.nb ? ib : 0u;
    const uint32_t flA = w.bflags[ca], flB = w.bflags[cb], bgA = w.bgen[ca], bgB = w.bgen[cb];
    const float imA = w.mat[ca].x, imB = w.mat[cb].x;
    const float4 iA = w.iinv[ca], iB = w.iinv[cb];
    const float4 qA4 = w.cur.rot[ca], qB4 = w.cur.rot[cb];
    const float4 lA4 = w.nxt.lin[ca], aA4 = w.nxt.ang[ca], lB4 = w.nxt.lin[cb], aB4 = w.nxt.ang[cb];

    // Cache range for (bodyA, bodyB); generations must match.
    const unsigned long long gens = ((unsigned long long)t.gA << 32) | t.gB;
    const uint2 rr = range ? *range : cacheRange(cacheKeys, cacheN, ia, ib);
    uint32_t rb = rr.x, re = rr.y;
    float4 preA[4], preB[4];
    float preT[4];
    unsigned long long gen0 = 0;
    if (rb < re) gen0 = a.oldCache.gens[rb];
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (rb + j < re) {
            preA[j] = a.oldCache.anchorA[rb + j];
            preB[j] = a.oldCache.anchorB[rb + j];
            preT[j] = a.oldCache.tangent2[rb + j];
        }

    const float4 nf = t.nf;
    const V3 n{nf.x, nf.y, nf.z};
    // A manifold whose body handles are stale is not solved and not cached
    // (sequential_impulse_solver.cpp:317-320).
    const bool valid = ia < w.nb && ib < w.nb && (flA & kBodyAlive) && (flB & kBodyAlive) && bgA == t.gA &&
                       bgB == t.gB && solvedPair(w, flA, flB);
    const bool sA = (flA & kBodyStatic) != 0, sB = (flB & kBodyStatic) != 0;
    const Q qA = f4q(qA4), qB = f4q(qB4);
    const M3 IA = inverseInertiaWorld(qA, iA.x, iA.y, iA.z);
    const M3 IB = inverseInertiaWorld(qB, iB.x, iB.y, iB.z);
    if (p == 0) {
        a.sb.pbody[k] = make_uint2(valid ? ia : 0u, valid ? ib : 0u);
        a.sb.pn[k] = nf;
        if (!valid) {
            a.sb.pcount[k] = 0;
            a.sb.pm[k] = make_float4(0.0f, 1.0f, 0.0f, 1.0f);
            return;  // no live points: nothing is solved or written back
        }
        ++tally.solved;
        a.sb.pcount[k] = live;
        a.sb.pm[k] = make_float4(imA, sA ? 1.0f : 0.0f, imB, sB ? 1.0f : 0.0f);
        a.sb.pmInertia[0 * mcap + k] = make_float4(IA.m00, IA.m01, IA.m02, 0.0f);
        a.sb.pmInertia[1 * mcap + k] = make_float4(IA.m10, IA.m11, IA.m12, 0.0f);
        a.sb.pmInertia[2 * mcap + k] = make_float4(IA.m20, IA.m21, IA.m22, 0.0f);
        a.sb.pmInertia[3 * mcap + k] = make_float4(IB.m00, IB.m01, IB.m02, 0.0f);
        a.sb.pmInertia[4 * mcap + k] = make_float4(IB.m10, IB.m11, IB.m12, 0.0f);
        a.sb.pmInertia[5 * mcap + k] = make_float4(IB.m20, IB.m21, IB.m22, 0.0f);
        if (live == 0) return;
    } else if (!valid) {
        return;
    }
    if (rb < re && gen0 != gens) re = rb;
    const V3 linA = f4xyz(lA4), angA = f4xyz(aA4);
    const V3 linB = f4xyz(lB4), angB = f4xyz(aB4);

    float4 out[kPreparedVec4];
    for (int v = 0; v < kPreparedVec4; ++v) out[v] = make_float4(0, 0, 0, 0);
    float4 imp = t.imp;
    imp.w = 0.0f;
    const V3 anchorA{t.aa.x, t.aa.y, t.aa.z}, anchorB{t.ab.x, t.ab.y, t.ab.z};
    const float penetration = t.aa.w;
    V3 offA = rotate(qA, anchorA), offB = rotate(qB, anchorB);
    out[0] = make4(offA, 0.0f);
    out[1] = make4(offB, 0.0f);
    V3 tref = fabsf(n.x) < 0.9f ? V3{1.0f, 0.0f, 0.0f} : V3{0.0f, 1.0f, 0.0f};
    V3 t1 = cross(n, tref);
    float tl = sqrtf(dot(t1, t1));
    if (tl > 1e-6f) {
        t1 = t1 / tl;
        V3 t2 = cross(n, t1);
        V3 vA = linA + cross(angA, offA), vB = linB + cross(angB, offB);
        float vin = dot(vB - vA, n);
        V3 jA = cross(offA, n), jB = cross(offB, n);
        V3 nrA = mul(IA, jA), nrB = mul(IB, jB);
        float ims = imA + imB;
        float iem = ims + dot(jA, nrA) + dot(jB, nrB);
        V3 tjA = cross(offA, t1), tjB = cross(offB, t1);
        V3 trA1 = mul(IA, tjA), trB1 = mul(IB, tjB);
        float tm00 = ims + dot(tjA, trA1) + dot(tjB, trB1);
        float ntr1 = ims * dot(n, t1) + dot(tjA, nrA) + dot(tjB, nrB);
        tjA = cross(offA, t2);
        tjB = cross(offB, t2);
        V3 trA2 = mul(IA, tjA), trB2 = mul(IB, tjB);
        float tm11 = ims + dot(tjA, trA2) + dot(tjB, trB2);
        float ntr2 = ims * dot(n, t2) + dot(tjA, nrA) + dot(tjB, nrB);
        float tm01 = dot(tjA, trA1) + dot(tjB, trB1);
        float det = tm00 * tm11 - tm01 * tm01;
        float itm00 = 0.0f, itm01 = 0.0f, itm11 = 0.0f;
        if (det > 0.0f) {
            float inv = 1.0f / det;
            itm00 = tm11 * inv;
            itm01 = -tm01 * inv;
            itm11 = tm00 * inv;
        }
        float bias = 0.0f, rv = 0.0f;
        if (!(iem <= 0.0f)) {
            ++tally.prepared;
            bias = smax(penetration - 0.005f, 0.0f) * (0.2f * (1.0f / smax(w.dt, 1e-6f)));
            rv = vin < -1.0f ? t.rest * vin : 0.0f;
        }
        out[0].w = iem;
        out[1].w = bias;
        out[2] = make4(t1, rv);
        out[3] = make4(t2, itm00);
        out[4] = make4(nrA, itm01);
        out[5] = make4(nrB, itm11);
        out[6] = make4(trA1, ntr1);
        out[7] = make4(trB1, ntr2);
        out[8] = make4(trA2, 0.0f);
        out[9] = make4(trB2, 0.0f);
        if (!(iem <= 0.0f)) {
            // first entry within 0.05 of both anchors (the range in cache order)
            const float matchSq = 0.05f * 0.05f;
            bool found = false;
            auto tryEntry = [&](const float4 &ca, const float4 &cb, float t2c) {
                ++tally.comparisons;
                V3 da = V3{ca.x, ca.y, ca.z} - anchorA, db = V3{cb.x, cb.y, cb.z} - anchorB;
                if (dot(da, da) > matchSq || dot(db, db) > matchSq) return;
                float ni = smax(ca.w, 0.0f);
                float limit = smax(nf.w, 0.0f) * ni;
                float tlsq = cb.w * cb.w + t2c * t2c;
                float scale = tlsq > limit * limit ? limit / sqrtf(tlsq) : 1.0f;
                imp = make_float4(ni, cb.w * scale, t2c * scale, 1.0f);
                ++tally.matches;
                found = true;
            };
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (!found && rb + j < re) tryEntry(preA[j], preB[j], preT[j]);
            for (uint32_t c = rb + 4; !found && c < re; ++c)
                tryEntry(a.oldCache.anchorA[c], a.oldCache.anchorB[c], a.oldCache.tangent2[c]);
        }
    }
    for (int v = 0; v < kPreparedVec4; ++v) a.sb.pp[(size_t)(v * 4 + p) * mcap + k] = out[v];
    a.sb.pimp[(size_t)p * mcap + k] = imp;
}

__device__ inline void prepareRange(const SolveArgs &a, uint32_t begin, uint32_t stride, uint32_t M,
                                    const unsigned long long *cacheKeys = nullptr) {
    if (!cacheKeys) cacheKeys = a.oldCache.key;
    const uint32_t cacheN = *a.oldCount;
    PrepTally tally;
    for (uint32_t q = begin; q < 4 * M; q += stride) prepareItem(a, loadPrepItem(a, q, M), cacheKeys, cacheN, tally);
    flushPrepTally(a, tally);
}


// ---------------------------------------------------------- solve sweeps ---
// Where the sweeps read a manifold's prepared data: the solver arrays by
// manifold index (GlobalPrep), or shared-memory copies by a local index.
struct GlobalPrep {
    const SolveArgs &a;
    __device__ __forceinline__ float4 pm(uint32_t i) const { return a.sb.pm[i]; }
    __device__ __forceinline__ float4 pn(uint32_t i) const { return a.sb.pn[i]; }
    __device__ __forceinline__ uint32_t count(uint32_t i) const { return a.sb.pcount[i]; }
    __device__ __forceinline__ float4 inertia(int r, uint32_t i) const { return a.sb.pmInertia[(size_t)r * a.mcap + i]; }
    __device__ __forceinline__ float4 pt(int v, uint32_t p, uint32_t i) const {
        return a.sb.pp[(size_t)(v * 4 + p) * a.mcap + i];
    }
    __device__ __forceinline__ float4 imp(uint32_t p, uint32_t i) const { return a.sb.pimp[(size_t)p * a.mcap + i]; }
    __device__ __forceinline__ void setImp(uint32_t p, uint32_t i, const float4 &v) const {
        a.sb.pimp[(size_t)p * a.mcap + i] = v;
    }
};

// Warm start of one manifold (warmStartPrepared's application, :491-517).  k:
// solve index (velocity slots), i: data index (prepared data).  Point 0's data
// are requested together with the manifold's, so a one-point manifold costs
// one memory round trip.
template <class Prep, class Vel>
__device__ __forceinline__ void warmStartOne(const Prep &pr, uint32_t k, uint32_t i, const Vel &vel) {
    const uint2 bi = vel.bodies(k, i);
    const float4 pm = pr.pm(i);
    const float4 nf = pr.pn(i);
    const uint32_t npts = pr.count(i);
    float4 r[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) r[j] = pr.inertia(j, i);
    float4 imp = pr.imp(0, i);
    float4 offA4 = pr.pt(0, 0, i), offB4 = pr.pt(1, 0, i), t14 = pr.pt(2, 0, i), t24 = pr.pt(3, 0, i);
    const bool sA = pm.y != 0.0f, sB = pm.w != 0.0f;
    const V3 n{nf.x, nf.y, nf.z};
    const M3 IA{r[0].x, r[0].y, r[0].z, r[1].x, r[1].y, r[1].z, r[2].x, r[2].y, r[2].z};
    const M3 IB{r[3].x, r[3].y, r[3].z, r[4].x, r[4].y, r[4].z, r[5].x, r[5].y, r[5].z};
    V3 linA = vel.lin(bi.x), angA = vel.ang(bi.x);
    V3 linB = vel.lin(bi.y), angB = vel.ang(bi.y);
    bool any = false;
    for (uint32_t p = 0; p < npts; ++p) {
        if (p > 0) {
            imp = pr.imp(p, i);
            offA4 = pr.pt(0, p, i);
            offB4 = pr.pt(1, p, i);
            t14 = pr.pt(2, p, i);
            t24 = pr.pt(3, p, i);
        }
        if (imp.w == 0.0f) continue;
        V3 wi = n * imp.x + f4xyz(t14) * imp.y + f4xyz(t24) * imp.z;
        V3 nw = -wi;
        if (!sA) {
            linA += nw * pm.x;
            angA += mul(IA, cross(f4xyz(offA4), nw));
        }
        if (!sB) {
            linB += wi * pm.z;
            angB += mul(IB, cross(f4xyz(offB4), wi));
        }
        any = true;
    }
    if (!any) return;
    if (!sA) vel.store(bi.x, linA, angA);
    if (!sB) vel.store(bi.y, linB, angB);
}
template <class Vel> __device__ __forceinline__ void warmStartOne(const SolveArgs &a, uint32_t k, uint32_t m, const Vel &vel) {
    warmStartOne(GlobalPrep{a}, k, m, vel);
}
__device__ __forceinline__ void warmStartOne(const SolveArgs &a, uint32_t k, uint32_t m) {
    warmStartOne(GlobalPrep{a}, k, m, GlobalVel{a});
}

// solvePrepared (:520-603) for one manifold; k, i as for warmStartOne.
template <class Prep, class Vel>
__device__ __forceinline__ void solveOne(const Prep &pr, uint32_t k, uint32_t i, const Vel &vel) {
    const uint2 bi = vel.bodies(k, i);
    const float4 pm = pr.pm(i);
    const float4 nf = pr.pn(i);
    const uint32_t npts = pr.count(i);
    // Point 0's constants come with the manifold's (one memory round trip);
    // further points load theirs in turn.
    float4 o[10];
#pragma unroll
    for (int v = 0; v < 10; ++v) o[v] = pr.pt(v, 0, i);
    float4 imp = pr.imp(0, i);
    const bool sA = pm.y != 0.0f, sB = pm.w != 0.0f;
    const V3 n{nf.x, nf.y, nf.z};
    const float friction = nf.w;
    V3 linA = vel.lin(bi.x), angA = vel.ang(bi.x);
    V3 linB = vel.lin(bi.y), angB = vel.ang(bi.y);
    for (uint32_t p = 0; p < npts; ++p) {
        if (p > 0) {
#pragma unroll
            for (int v = 0; v < 10; ++v) o[v] = pr.pt(v, p, i);
            imp = pr.imp(p, i);
        }
        if (o[0].w <= 0.0f) continue;  // inverseEffectiveMass <= 0
        const V3 offA = f4xyz(o[0]), offB = f4xyz(o[1]), t1 = f4xyz(o[2]), t2 = f4xyz(o[3]);
        const float iem = o[0].w, bias = o[1].w, rv = o[2].w, itm00 = o[3].w, itm01 = o[4].w, itm11 = o[5].w;
        const V3 vA = linA + cross(angA, offA);
        const V3 vB = linB + cross(angB, offB);
        const V3 rel = vB - vA;
        float vn = dot(rel, n);
        float delta = -(vn + rv - bias) / iem;
        float prev = imp.x;
        imp.x = smax(prev + delta, 0.0f);
        float applied = imp.x - prev;
        V3 impulse = n * applied;
        if (!sA) {
            linA += (-impulse) * pm.x;
            angA += f4xyz(o[4]) * (-applied);
        }
        if (!sB) {
            linB += impulse * pm.z;
            angB += f4xyz(o[5]) * applied;
        }
        if (itm00 <= 0.0f || itm11 <= 0.0f) {
            pr.setImp(p, i, imp);
            continue;
        }
        const float ntr1 = o[6].w, ntr2 = o[7].w;
        float limit = smax(friction, 0.0f) * imp.x;
        float tv1 = dot(rel, t1) + ntr1 * applied;
        float tv2 = dot(rel, t2) + ntr2 * applied;
        float d1 = -(itm00 * tv1 + itm01 * tv2);
        float d2 = -(itm01 * tv1 + itm11 * tv2);
        float p1 = imp.y, p2 = imp.z;
        imp.y += d1;
        imp.z += d2;
        float lsq = imp.y * imp.y + imp.z * imp.z;
        if (lsq > limit * limit) {
            float sc = limit / sqrtf(lsq);
            imp.y *= sc;
            imp.z *= sc;
        }
        float a1 = imp.y - p1, a2 = imp.z - p2;
        V3 ti = t1 * a1 + t2 * a2;
        V3 rA = f4xyz(o[6]) * a1 + f4xyz(o[8]) * a2;
        V3 rB = f4xyz(o[7]) * a1 + f4xyz(o[9]) * a2;
        if (!sA) {
            linA += (-ti) * pm.x;
            angA += -rA;
        }
        if (!sB) {
            linB += ti * pm.z;
            angB += rB;
        }
        pr.setImp(p, i, imp);
    }
    if (!sA) vel.store(bi.x, linA, angA);
    if (!sB) vel.store(bi.y, linB, angB);
}
// solveOne for prepared data read from L2 (the island sweeps of the
// multi-kernel path): each further point's constants are requested while the
// point before it is solved (they do not depend on it), so only the first load
// is on the update chain.  The arithmetic is solveOne's, operation for operation.
template <class Prep, class Vel>
__device__ __forceinline__ void solveOneChained(const Prep &pr, uint32_t k, uint32_t i, const Vel &vel) {
    const uint2 bi = vel.bodies(k, i);
    const float4 pm = pr.pm(i);
    const float4 nf = pr.pn(i);
    const uint32_t npts = pr.count(i);
    float4 o[10], on[10];
#pragma unroll
    for (int v = 0; v < 10; ++v) o[v] = pr.pt(v, 0, i);
    float4 imp = pr.imp(0, i), impn = imp;
    const bool sA = pm.y != 0.0f, sB = pm.w != 0.0f;
    const V3 n{nf.x, nf.y, nf.z};
    const float friction = nf.w;
    V3 linA = vel.lin(bi.x), angA = vel.ang(bi.x);
    V3 linB = vel.lin(bi.y), angB = vel.ang(bi.y);
    for (uint32_t p = 0; p < npts; ++p) {
        if (p > 0) {
#pragma unroll
            for (int v = 0; v < 10; ++v) o[v] = on[v];
            imp = impn;
        }
        if (p + 1 < npts) {
#pragma unroll
            for (int v = 0; v < 10; ++v) on[v] = pr.pt(v, p + 1, i);
            impn = pr.imp(p + 1, i);
        }
        if (o[0].w <= 0.0f) continue;  // inverseEffectiveMass <= 0
        const V3 offA = f4xyz(o[0]), offB = f4xyz(o[1]), t1 = f4xyz(o[2]), t2 = f4xyz(o[3]);
        const float iem = o[0].w, bias = o[1].w, rv = o[2].w, itm00 = o[3].w, itm01 = o[4].w, itm11 = o[5].w;
        const V3 vA = linA + cross(angA, offA);
        const V3 vB = linB + cross(angB, offB);
        const V3 rel = vB - vA;
        float vn = dot(rel, n);
        float delta = -(vn + rv - bias) / iem;
        float prev = imp.x;
        imp.x = smax(prev + delta, 0.0f);
        float applied = imp.x - prev;
        V3 impulse = n * applied;
        if (!sA) {
            linA += (-impulse) * pm.x;
            angA += f4xyz(o[4]) * (-applied);
        }
        if (!sB) {
            linB += impulse * pm.z;
            angB += f4xyz(o[5]) * applied;
        }
        if (itm00 <= 0.0f || itm11 <= 0.0f) {
            pr.setImp(p, i, imp);
            continue;
        }
        const float ntr1 = o[6].w, ntr2 = o[7].w;
        float limit = smax(friction, 0.0f) * imp.x;
        float tv1 = dot(rel, t1) + ntr1 * applied;
        float tv2 = dot(rel, t2) + ntr2 * applied;
        float d1 = -(itm00 * tv1 + itm01 * tv2);
        float d2 = -(itm01 * tv1 + itm11 * tv2);
        float p1 = imp.y, p2 = imp.z;
        imp.y += d1;
        imp.z += d2;
        float lsq = imp.y * imp.y + imp.z * imp.z;
        if (lsq > limit * limit) {
            float sc = limit / sqrtf(lsq);
            imp.y *= sc;
            imp.z *= sc;
        }
        float a1 = imp.y - p1, a2 = imp.z - p2;
        V3 ti = t1 * a1 + t2 * a2;
        V3 rA = f4xyz(o[6]) * a1 + f4xyz(o[8]) * a2;
        V3 rB = f4xyz(o[7]) * a1 + f4xyz(o[9]) * a2;
        if (!sA) {
            linA += (-ti) * pm.x;
            angA += -rA;
        }
        if (!sB) {
            linB += ti * pm.z;
            angB += rB;
        }
        pr.setImp(p, i, imp);
    }
    if (!sA) vel.store(bi.x, linA, angA);
    if (!sB) vel.store(bi.y, linB, angB);
}
template <class Vel> __device__ __forceinline__ void solveOne(const SolveArgs &a, uint32_t k, uint32_t m, const Vel &vel) {
    solveOne(GlobalPrep{a}, k, m, vel);
}
__device__ __forceinline__ void solveOne(const SolveArgs &a, uint32_t k, uint32_t m) {
    solveOne(GlobalPrep{a}, k, m, GlobalVel{a});
}
__device__ __forceinline__ void solveOneChained(const SolveArgs &a, uint32_t k, uint32_t m) {
    solveOneChained(GlobalPrep{a}, k, m, GlobalVel{a});
}

__device__ __forceinline__ void cacheWriteManifold(const SolveArgs &a, const CacheView &nc, uint32_t cacheCap,
                                                   uint32_t m, uint32_t base, uint32_t npts) {
    const unsigned long long key = ((unsigned long long)a.mv.bodyA[m] << 32) | a.mv.bodyB[m];
    const unsigned long long gens = ((unsigned long long)a.mv.genA[m] << 32) | a.mv.genB[m];
    for (uint32_t p = 0; p < npts; ++p) {
        const uint32_t e = base + p;
        if (e >= cacheCap) break;
        const float4 aa = a.mv.anchorA[4 * m + p], ab = a.mv.anchorB[4 * m + p];
        const float4 imp = __ldcg(&a.mv.impulse[4 * m + p]);  // may come from other SMs of a cluster
        nc.key[e] = key;
        nc.gens[e] = gens;
        nc.anchorA[e] = make_float4(aa.x, aa.y, aa.z, imp.x);
        nc.anchorB[e] = make_float4(ab.x, ab.y, ab.z, imp.y);
        nc.tangent2[e] = imp.z;
    }
}


// The manifold's body handles are live (sequential_impulse_solver.cpp:317-320).
__device__ __forceinline__ bool manifoldBodiesValid(const SolveArgs &a, uint32_t m) {
    const uint32_t ia = a.mv.bodyA[m], ib = a.mv.bodyB[m];
    const WorldView &w = a.w;
    return ia < w.nb && ib < w.nb && (w.bflags[ia] & kBodyAlive) && (w.bflags[ib] & kBodyAlive) &&
           w.bgen[ia] == a.mv.genA[m] && w.bgen[ib] == a.mv.genB[m] && solvedPair(w, w.bflags[ia], w.bflags[ib]);
}

// Per-manifold body flags: bit 0 / bit 1 body A / B live, of the manifold's
// generation and dynamic (the colouring's "dynamic side"); bit 2 both handles
// live (the manifold is solved).
constexpr uint32_t kFlagDynA = 1u, kFlagDynB = 2u, kFlagValid = 4u;
__device__ __forceinline__ uint32_t manifoldFlagsOf(const WorldView &w, uint32_t ba, uint32_t bb, uint32_t genA,
                                                    uint32_t genB) {
    const bool okA = ba < w.nb && (w.bflags[ba] & kBodyAlive) && w.bgen[ba] == genA;
    const bool okB = bb < w.nb && (w.bflags[bb] & kBodyAlive) && w.bgen[bb] == genB;
    const bool dA = okA && !(w.bflags[ba] & (kBodyStatic | kBodySleeping));
    const bool dB = okB && !(w.bflags[bb] & (kBodyStatic | kBodySleeping));
    return (dA ? kFlagDynA : 0u) | (dB ? kFlagDynB : 0u) |
           (okA && okB && (!w.sleepMode || dA || dB) ? kFlagValid : 0u);
}
__device__ __forceinline__ uint32_t manifoldFlags(const SolveArgs &a, uint32_t m) {
    return manifoldFlagsOf(a.w, a.mv.bodyA[m], a.mv.bodyB[m], a.mv.genA[m], a.mv.genB[m]);
}

// Front of the single-block solver: staging slots, colouring and the solve
// order.  Afterwards sb.order and s_dyn map solve index k to manifold m (colour
// path; the reference order is the identity), sh.start / sh.colors hold the
// colour ranges and, when it returns true, vs->slot[k] the staging slots of
// solve index k's bodies and vs->slotBody / sh.slots the staged bodies.
// mflags: manifoldFlags of every manifold, written by an earlier launch or
// cluster rank (nullptr: computed here).
__device__ inline bool solveBlockFront(const SolveArgs &a, uint32_t M, int serial, uint32_t maxM,
                                       unsigned long long *s_sort, uint32_t *s_dyn, BlockSolveShared &sh,
                                       const VelStage *vs, const uint32_t *mflags = nullptr) {
    uint32_t *s_start = sh.start, *s_count = sh.count, *s_scan = sh.scan;
    uint32_t &s_colored = sh.colored, &s_colors = sh.colors;
    const WorldView &w = a.w;
    const SolverBuffers &sb = a.sb;
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    bool slotted = false;  // bodies got staging slots (colour path with a VelStage)
    if (serial) {
        for (uint32_t k = tid; k < M; k += nt) sb.order[k] = k;
        __syncthreads();
    } else {
        // --- body flags of every manifold (s_dyn until the placement) ---
        for (uint32_t m = tid; m < M; m += nt) s_dyn[m] = mflags ? __ldcg(&mflags[m]) : manifoldFlags(a, m);
        __syncthreads();
        // --- staging slots for the bodies of valid manifolds, assigned through a
        // shared-memory hash table (in the velocity area, free until the
        // colouring); the colouring's per-body arrays and, after prepare, the
        // staged velocities use them ---
        if (vs) {
            uint32_t *tkey = reinterpret_cast<uint32_t *>(vs->v);
            // at most 2M keys: a table of >= 4M entries (load <= 1/2) where the
            // key and value words fit the velocity area's 8 words per slot
            uint32_t T = 32;
            while (T < 4 * M && 2 * T <= 4 * vs->cap) T <<= 1;
            uint32_t *tval = tkey + T;
            for (uint32_t i = tid; i < T; i += nt) tkey[i] = kSlotFree;
            if (tid == 0) {
                sh.slots = 0;
                sh.colored = 0;  // table overflow flag until the colouring starts
            }
            __syncthreads();
            for (uint32_t m = tid; m < M; m += nt) {
                if (!(s_dyn[m] & kFlagValid)) continue;
                const uint32_t b2[2] = {a.mv.bodyA[m], a.mv.bodyB[m]};
                for (int j = 0; j < 2; ++j) {
                    uint32_t h = (b2[j] * 2654435761u) & (T - 1), probes = 0;
                    for (;; h = (h + 1) & (T - 1)) {
                        const uint32_t old = atomicCAS(&tkey[h], kSlotFree, b2[j]);
                        if (old == kSlotFree || old == b2[j]) break;
                        if (++probes == T) {
                            sh.colored = 1;
                            break;
                        }
                    }
                }
            }
            __syncthreads();
            for (uint32_t i = tid; i < T; i += nt) {  // T is a multiple of 32: whole warps
                const uint32_t key = tkey[i];
                const uint32_t lane = tid & 31;
                const uint32_t used = __ballot_sync(0xffffffffu, key != kSlotFree);
                uint32_t base = 0;
                if (lane == 0 && used) base = atomicAdd(&sh.slots, (uint32_t)__popc(used));
                base = __shfl_sync(0xffffffffu, base, 0);
                if (key == kSlotFree) continue;
                const uint32_t sl = base + __popc(used & ((1u << lane) - 1u));
                tval[i] = sl;
                if (sl < vs->cap) vs->slotBody[sl] = key;
            }
            __syncthreads();
            slotted = sh.colored == 0 && sh.slots <= vs->cap;
            if (slotted) {
                auto find = [&](uint32_t body) {
                    uint32_t h = (body * 2654435761u) & (T - 1);
                    for (uint32_t probes = 0; probes < T && tkey[h] != body; ++probes) h = (h + 1) & (T - 1);
                    return tval[h];
                };
                for (uint32_t m = tid; m < M; m += nt)
                    vs->slot[m] = (s_dyn[m] & kFlagValid) ? make_uint2(find(a.mv.bodyA[m]), find(a.mv.bodyB[m]))
                                                          : make_uint2(0u, 0u);
                __syncthreads();  // the colouring arrays below overwrite the table
                unsigned long long *best = reinterpret_cast<unsigned long long *>(vs->v);
                for (uint32_t sl = tid; sl < 3 * sh.slots; sl += nt) best[sl < sh.slots ? sl : vs->cap + (sl - sh.slots)] = 0ull;
            }
            __syncthreads();
        }
        // --- colouring (Jones-Plassmann rounds in colour windows, as k_color);
        // per-body arrays in shared memory by slot when slotted, else in global
        // memory by body ---
        for (uint32_t c = tid; c < kMaxColors; c += nt) s_count[c] = 0;
        if (tid == 0) {
            s_colored = 0;
            s_colors = 0;
            sh.deferred = 0;
        }
        unsigned long long *cBest = sb.bodyBest, *cUsed = sb.bodyUsed;
        if (slotted) {
            cBest = reinterpret_cast<unsigned long long *>(vs->v);
            cUsed = cBest + vs->cap;
        }
        auto cid = [&](uint32_t m, int side) -> uint32_t {
            return slotted ? (side ? vs->slot[m].y : vs->slot[m].x) : (side ? a.mv.bodyB[m] : a.mv.bodyA[m]);
        };
        // Atomics resolve in L2; global reads go past L1 so no stale line is seen.
        auto ldc = [&](const unsigned long long *p) { return slotted ? *p : __ldcg(p); };
        auto stc = [&](unsigned long long *p, unsigned long long v) {
            if (slotted) *p = v;
            else __stcg(p, v);
        };
        uint32_t *s_color = reinterpret_cast<uint32_t *>(s_sort);  // reused before the order sort
        for (uint32_t m = tid; m < M; m += nt) {
            const uint32_t fl = s_dyn[m];
            const bool da = fl & kFlagDynA, db = fl & kFlagDynB;
            s_color[m] = kUncolored;
            if (!slotted) {
                const uint32_t ba = a.mv.bodyA[m], bb = a.mv.bodyB[m];
                if (da) {
                    __stcg(&sb.bodyUsed[2 * ba], 0ull);
                    __stcg(&sb.bodyUsed[2 * ba + 1], 0ull);
                }
                if (db) {
                    __stcg(&sb.bodyUsed[2 * bb], 0ull);
                    __stcg(&sb.bodyUsed[2 * bb + 1], 0ull);
                }
            }
        }
        __syncthreads();
        const unsigned long long epoch0 = __ldcg(sb.epoch);
        uint32_t rounds = 0, base = 0;
        bool exhausted = false;
        for (;;) {  // one colour window [base, base + kMaxColors) per pass
            uint32_t round = 0;
            for (; round < kMaxRounds; ++round) {
                const unsigned long long stamp = (epoch0 + rounds + round + 1) << 32;
                for (uint32_t m = tid; m < M; m += nt) {
                    if (s_color[m] != kUncolored) continue;
                    const unsigned long long p = stamp | colorPriority(m);
                    if (s_dyn[m] & 1u) atomicMax(&cBest[cid(m, 0)], p);
                    if (s_dyn[m] & 2u) atomicMax(&cBest[cid(m, 1)], p);
                }
                __syncthreads();
                // (m0 advances uniformly so that whole warps aggregate the counters)
                for (uint32_t m0 = 0; m0 < M; m0 += nt) {
                    const uint32_t m = m0 + tid;
                    uint32_t c = kUncolored;
                    if (m < M && s_color[m] == kUncolored) {
                        const unsigned long long p = stamp | colorPriority(m);
                        const uint32_t d = s_dyn[m], ba = cid(m, 0), bb = cid(m, 1);
                        const bool wins =
                            (!(d & 1u) || ldc(&cBest[ba]) == p) && (!(d & 2u) || ldc(&cBest[bb]) == p);
                        if (wins) {
                            unsigned long long u0 = 0, u1 = 0;
                            if (d & 1u) {
                                u0 |= ldc(&cUsed[2 * ba]);
                                u1 |= ldc(&cUsed[2 * ba + 1]);
                            }
                            if (d & 2u) {
                                u0 |= ldc(&cUsed[2 * bb]);
                                u1 |= ldc(&cUsed[2 * bb + 1]);
                            }
                            uint32_t local = kDeferred;
                            if (~u0) local = __ffsll((long long)~u0) - 1;
                            else if (~u1) local = 64 + __ffsll((long long)~u1) - 1;
                            if (local != kDeferred) {
                                c = base + local;
                                const unsigned long long bit = 1ull << (local & 63);
                                if (d & 1u) stc(&cUsed[2 * ba + (local >> 6)], ldc(&cUsed[2 * ba + (local >> 6)]) | bit);
                                if (d & 2u) stc(&cUsed[2 * bb + (local >> 6)], ldc(&cUsed[2 * bb + (local >> 6)]) | bit);
                            } else {
                                c = kDeferred;
                            }
                            s_color[m] = c;
                        }
                    }
                    // one shared-memory atomic per warp and counter
                    const uint32_t lane = tid & 31;
                    const bool done = c != kUncolored, got = done && c != kDeferred;
                    const uint32_t doneMask = __ballot_sync(0xffffffffu, done);
                    const uint32_t gotMask = __ballot_sync(0xffffffffu, got);
                    const uint32_t top = __reduce_max_sync(0xffffffffu, got ? c + 1 : 0u);
                    if (lane == 0 && doneMask) {
                        atomicAdd(&s_colored, (uint32_t)__popc(doneMask));
                        if (doneMask != gotMask) atomicAdd(&sh.deferred, (uint32_t)__popc(doneMask & ~gotMask));
                        if (gotMask) atomicMax(&s_colors, top);
                    }
                    const uint32_t peers = __match_any_sync(0xffffffffu, c);
                    if (got && c < (uint32_t)kMaxColors && (peers & ((1u << lane) - 1u)) == 0)
                        atomicAdd(&s_count[c], (uint32_t)__popc(peers));
                }
                __syncthreads();
                if (s_colored >= M) break;
                __syncthreads();
            }
            rounds += round + 1;
            if (round >= kMaxRounds) {
                exhausted = true;
                break;
            }
            const uint32_t deferred = sh.deferred;
            __syncthreads();
            if (deferred == 0) break;
            // next window: the deferred manifolds become uncoloured again and
            // the masks of their bodies start empty
            base += kMaxColors;
            for (uint32_t m = tid; m < M; m += nt) {
                if (s_color[m] != kDeferred) continue;
                s_color[m] = kUncolored;
                const uint32_t d = s_dyn[m];
                for (int e = 0; e < 2; ++e)
                    if (d & (1u << e)) {
                        stc(&cUsed[2 * cid(m, e)], 0ull);
                        stc(&cUsed[2 * cid(m, e) + 1], 0ull);
                    }
            }
            if (tid == 0) {
                s_colored = M - deferred;
                sh.deferred = 0;
            }
            __syncthreads();
        }
        if (exhausted) {
            // The step fails (kErrColors); colour 0 for what is left keeps every
            // index below in range.
            for (uint32_t m = tid; m < M; m += nt)
                if (s_color[m] >= kDeferred) s_color[m] = 0;
            if (tid == 0 && s_colors == 0) s_colors = 1;
            __syncthreads();
        }
        if (tid == 0) {
            *sb.epoch = epoch0 + rounds + 2;
            a.st->colorRounds = rounds;
            a.st->colors = s_colors;
            if (exhausted) atomicOr(&a.st->err, kErrColors);
            if (s_colors <= (uint32_t)kMaxColors) {
                uint32_t acc = 0;
                for (uint32_t c = 0; c < s_colors; ++c) {
                    s_start[c] = acc;
                    sb.colorCount[c] = s_count[c];
                    acc += s_count[c];
                }
                s_start[s_colors] = acc;
            }
        }
        // colours to global (pair order) and the (colour, index) order
        for (uint32_t m = tid; m < M; m += nt) sb.color[m] = s_color[m];
        __syncthreads();
        const uint32_t nw = nt >> 5, Cc = s_colors;
        if (Cc <= (uint32_t)kMaxColors && nw * Cc <= 2 * maxM) {
            // Stable placement: a manifold goes to the start of its colour plus
            // the number of earlier manifolds of that colour (warp ranks from
            // match_any, per-warp colour counts scanned across warps).
            uint32_t *wc = reinterpret_cast<uint32_t *>(s_sort);  // [warps][colours]
            const uint32_t lane = tid & 31, warp = tid >> 5;
            for (uint32_t c = tid; c < Cc; c += nt) s_count[c] = 0;
            for (uint32_t m0 = 0; m0 < M; m0 += nt) {
                for (uint32_t i = tid; i < nw * Cc; i += nt) wc[i] = 0;
                __syncthreads();
                const uint32_t m = m0 + tid;
                const uint32_t c = m < M ? __ldcg(&sb.color[m]) : 0xFFFFFFFFu;
                const uint32_t peers = __match_any_sync(0xffffffffu, c);
                const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
                if (m < M && rank == 0) wc[warp * Cc + c] = __popc(peers);
                __syncthreads();
                for (uint32_t cc = tid; cc < Cc; cc += nt) {
                    uint32_t run = s_count[cc];
                    for (uint32_t w2 = 0; w2 < nw; ++w2) {
                        const uint32_t t = wc[w2 * Cc + cc];
                        wc[w2 * Cc + cc] = run;
                        run += t;
                    }
                    s_count[cc] = run;
                }
                __syncthreads();
                if (m < M) {
                    const uint32_t k = s_start[c] + wc[warp * Cc + c] + rank;
                    sb.order[k] = m;
                    s_dyn[k] = m;  // solve index -> manifold for the sweeps
                }
                __syncthreads();
            }
        } else {
            const uint32_t n2 = nextPow2(M > 0 ? M : 1);
            uint32_t *keys = reinterpret_cast<uint32_t *>(s_sort);
            for (uint32_t i = tid; i < n2; i += nt) keys[i] = i < M ? ((sb.color[i] << 12) | i) : 0xFFFFFFFFu;
            __syncthreads();
            blockBitonicSort<uint32_t>(keys, n2);
            __syncthreads();  // s_dyn (colouring flags) is read no more
            for (uint32_t k = tid; k < M; k += nt) {
                sb.order[k] = keys[k] & 0xFFFu;
                s_dyn[k] = keys[k] & 0xFFFu;
                // more colours than the shared ranges hold: colour c starts at
                // sb.colorStart[c] (every colour below the last is used, so
                // each has a first solve index)
                if (Cc > (uint32_t)kMaxColors && (k == 0 || (keys[k] >> 12) != (keys[k - 1] >> 12)) &&
                    (keys[k] >> 12) < M)
                    sb.colorStart[keys[k] >> 12] = k;
            }
        }
        __syncthreads();
        if (slotted) {
            // slots by manifold -> slots by solve index (through the sort area)
            uint2 *tmp = reinterpret_cast<uint2 *>(s_sort);
            for (uint32_t k = tid; k < M; k += nt) tmp[k] = vs->slot[s_dyn[k]];
            __syncthreads();
            for (uint32_t k = tid; k < M; k += nt) vs->slot[k] = tmp[k];
            __syncthreads();
        }
    }
    return slotted;
}

// Warm-start cache rebuild (:623-681) of the single-block solver, after the
// impulses are back in the manifolds.
__device__ inline void solveBlockCache(const SolveArgs &a, const CacheView &nc, uint32_t cacheCap, uint32_t *newCount,
                                       uint32_t M, unsigned long long *s_sort, uint32_t *s_dyn, BlockSolveShared &sh) {
    uint32_t *s_scan = sh.scan;
    const WorldView &w = a.w;
    const SolverBuffers &sb = a.sb;
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    // --- cache rebuild ---
    if (a.pairOrderCache) {
        // Manifold order is (body A, body B) order with one manifold per key:
        // the cache is the manifolds' points in manifold order.
        for (uint32_t i = tid; i < M; i += nt) {
            const uint32_t ia = a.mv.bodyA[i], ib = a.mv.bodyB[i];
            const bool valid = ia < w.nb && ib < w.nb && (w.bflags[ia] & kBodyAlive) && (w.bflags[ib] & kBodyAlive) &&
                               w.bgen[ia] == a.mv.genA[i] && w.bgen[ib] == a.mv.genB[i] &&
                               solvedPair(w, w.bflags[ia], w.bflags[ib]);
            s_dyn[i] = valid ? min(a.mv.pointCount[i], 4u) : 0u;
        }
        __syncthreads();
        const uint32_t total = blockExclusiveScanArray(s_dyn, M, s_scan);
        for (uint32_t i = tid; i < M; i += nt) {
            const uint32_t cnt = (i + 1 < M ? s_dyn[i + 1] : total) - s_dyn[i];
            cacheWriteManifold(a, nc, cacheCap, i, s_dyn[i], cnt);
        }
        if (tid == 0) *newCount = total;
        return;
    }
    // stable sort by (body A, body B) over solve order
    const uint32_t n2 = nextPow2(M > 0 ? M : 1);
    for (uint32_t i = tid; i < n2; i += nt) {
        unsigned long long key = ~0ull;
        if (i < M) {
            const uint32_t m = sb.order[i];
            key = ((unsigned long long)a.mv.bodyA[m] << 44) | ((unsigned long long)a.mv.bodyB[m] << 24) | i;
        }
        s_sort[i] = key;
    }
    __syncthreads();
    blockBitonicSort<unsigned long long>(s_sort, n2);
    for (uint32_t i = tid; i < M; i += nt) {
        const uint32_t m = sb.order[(uint32_t)(s_sort[i] & 0xFFFu)];
        const uint32_t ia = a.mv.bodyA[m], ib = a.mv.bodyB[m];
        const bool valid = ia < w.nb && ib < w.nb && (w.bflags[ia] & kBodyAlive) && (w.bflags[ib] & kBodyAlive) &&
                           w.bgen[ia] == a.mv.genA[m] && w.bgen[ib] == a.mv.genB[m] &&
                           solvedPair(w, w.bflags[ia], w.bflags[ib]);
        s_dyn[i] = valid ? min(a.mv.pointCount[m], 4u) : 0u;
    }
    __syncthreads();
    const uint32_t total = blockExclusiveScanArray(s_dyn, M, s_scan);
    for (uint32_t i = tid; i < M; i += nt) {
        const uint32_t m = sb.order[(uint32_t)(s_sort[i] & 0xFFFu)];
        const uint32_t cnt = (i + 1 < M ? s_dyn[i + 1] : total) - s_dyn[i];
        cacheWriteManifold(a, nc, cacheCap, m, s_dyn[i], cnt);
    }
    if (tid == 0) *newCount = total;}

// Sweeps of the single-block solver after prepare: velocity staging (when
// slotted), warm start and iterations colour by colour, write-back, impulses
// back to the manifolds.
__device__ inline void solveBlockSweeps(const SolveArgs &a, uint32_t M, int serial, uint32_t C, bool slotted,
                                        const uint32_t *s_dyn, BlockSolveShared &sh, const VelStage *vs) {
    const uint32_t *s_start = sh.start;
    const WorldView &w = a.w;
    const SolverBuffers &sb = a.sb;
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    // --- stage the touched bodies' velocities in shared memory (slots from above) ---
    const bool staged = slotted;
    if (staged) {
        for (uint32_t sl = tid; sl < sh.slots; sl += nt) {
            const uint32_t b = vs->slotBody[sl];
            vs->v[2 * sl] = ld4(&w.nxt.lin[b]);
            vs->v[2 * sl + 1] = ld4(&w.nxt.ang[b]);
        }
        __syncthreads();
    }
    // --- warm start and velocity iterations ---
    // (manifold of solve index k: k itself in reference order, s_dyn[k] otherwise)
    if (serial) {
        if (tid == 0) {
            for (uint32_t k = 0; k < M; ++k) warmStartOne(a, k, k);
            for (int it = 0; it < a.iterations; ++it)
                for (uint32_t k = 0; k < M; ++k) solveOne(a, k, k);
        }
    } else if (staged) {
        const SharedVel sv{vs->v, vs->slot};
        for (uint32_t c = 0; c < C; ++c) {
            const uint2 r = colorRange(sh, sb, c, C, M);
            for (uint32_t k = r.x + tid; k < r.y; k += nt) warmStartOne(a, k, s_dyn[k], sv);
            __syncthreads();
        }
        for (int it = 0; it < a.iterations; ++it)
            for (uint32_t c = 0; c < C; ++c) {
                const uint2 r = colorRange(sh, sb, c, C, M);
                for (uint32_t k = r.x + tid; k < r.y; k += nt) solveOne(a, k, s_dyn[k], sv);
                __syncthreads();
            }
    } else {
        for (uint32_t c = 0; c < C; ++c) {
            const uint2 r = colorRange(sh, sb, c, C, M);
            for (uint32_t k = r.x + tid; k < r.y; k += nt) warmStartOne(a, k, s_dyn[k]);
            __syncthreads();
        }
        for (int it = 0; it < a.iterations; ++it)
            for (uint32_t c = 0; c < C; ++c) {
                const uint2 r = colorRange(sh, sb, c, C, M);
                for (uint32_t k = r.x + tid; k < r.y; k += nt) solveOne(a, k, s_dyn[k]);
                __syncthreads();
            }
    }
    __syncthreads();
    if (staged) {
        const uint32_t nslots = sh.slots;
        for (uint32_t sl = tid; sl < nslots; sl += nt) {
            const uint32_t b = vs->slotBody[sl];
            st4(&w.nxt.lin[b], vs->v[2 * sl]);
            st4(&w.nxt.ang[b], vs->v[2 * sl + 1]);
        }
        __syncthreads();
    }
    // --- impulses of the live points back to the manifolds ---
    for (uint32_t m = tid; m < M; m += nt) {
        const uint32_t live = sb.pcount[m];
        for (uint32_t p = 0; p < live; ++p) {
            float4 imp = sb.pimp[(size_t)p * a.mcap + m];
            imp.w = 0.0f;
            a.mv.impulse[4 * m + p] = imp;
        }
    }
    __syncthreads();
}

// ------------------------------------------------------ single-block path ---
// The whole solver for up to kBlockMaxManifolds manifolds in one thread block:
// the same colouring, order, prepare, sweeps and cache rebuild as the
// multi-kernel path, separated by __syncthreads instead of kernel boundaries
// and grid barriers.  If the live manifold count exceeds the block capacity the
// kernel only flags kErrSmallPath; the step is then re-run on the multi-kernel
// path.
// s_sort holds maxM u64 and s_dyn maxM u32 (shared memory); sh the small
// shared arrays.  prepared: the prepared data and the manifold flags (sb.dyn)
// were written by a launch before this one (else the block computes them
// itself).  All threads of the block call it.
__device__ inline void solveBlock(const SolveArgs &a, const CacheView &nc, uint32_t cacheCap, uint32_t *newCount, int serial,
                           uint32_t maxM, unsigned long long *s_sort, uint32_t *s_dyn, BlockSolveShared &sh,
                           const VelStage *vs = nullptr, bool prepared = false) {
    const uint32_t M = min(*a.count, a.mcap);
    if (M > maxM) {
        if (threadIdx.x == 0) atomicOr(&a.st->err, kErrSmallPath);
        return;
    }
    const uint32_t tid = threadIdx.x, nt = blockDim.x;
    const bool slotted = solveBlockFront(a, M, serial, maxM, s_sort, s_dyn, sh, vs, prepared ? a.sb.dyn : nullptr);
    const uint32_t C = serial ? 0u : sh.colors;
    // --- prepare + warm-start matching (old cache keys searched in shared memory when they fit) ---
    if (!prepared) {
        const uint32_t cacheN = *a.oldCount;
        const bool keysInShared = cacheN <= maxM;
        if (keysInShared)
            for (uint32_t i = tid; i < cacheN; i += nt) s_sort[i] = a.oldCache.key[i];
        __syncthreads();
        prepareRange(a, tid, nt, M, keysInShared ? s_sort : nullptr);
    }
    __syncthreads();
    solveBlockSweeps(a, M, serial, C, slotted, s_dyn, sh, vs);
    solveBlockCache(a, nc, cacheCap, newCount, M, s_sort, s_dyn, sh);
}


// The solver on one thread-block cluster (k_solve_cluster.cu): colour order
// only.  Returns false, launching nothing, when the device cannot run the
// cluster or the capacities do not fit its shared memory.
ClusterSolveLayout clusterSolveLayout(uint32_t blockM, uint32_t stageSlots);
bool launchSolverCluster(const SolveArgs &a, const CacheView &newCache, uint32_t *newCacheCount, uint32_t cacheCap,
                         uint32_t blockM, uint32_t stageSlots, cudaStream_t s);


} // namespace pe
