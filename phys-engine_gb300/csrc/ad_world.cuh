// Differentiable world step: PhysicsWorld::step (src/world/physics_world.cpp:
// 518-782) for a small world of sphere/box bodies, written for a team of
// threads (one CUDA thread block, or one host thread) over a scalar type S,
// plus its hand-written reverse (adjoint) with the contact set of the forward
// pass frozen: the pairs, the separating axes / kept vertices, the colour
// order, the warm-start matches and every clamp branch are the ones the
// forward evaluation took; everything continuous is differentiated, including
// the contact points, normals and depths as functions of the poses.
//
// Forward (mirrors the engine stage by stage): velocity integration, AABBs,
// all-pairs AABB test in lexicographic order (= the SAP pair set and order),
// narrowphase in pair order, greedy colouring by manifold priority (= the
// engine's colouring), solve order (colour, index), prepare + warm-start
// matching, warm start, velocity iterations, cache rebuild, pose integration.
//
// Reverse, per step, given the adjoints of the step's outputs (poses,
// velocities, and the final impulses that the next step's warm start read):
//   pose integration -> velocity iterations (colours in reverse, points in
//   reverse, from a tape of the pre-update velocities and impulses) -> warm
//   start -> warm-start matching (to the previous step's impulses) -> contact
//   geometry + preparation (forward-mode dual numbers, four directions at a
//   time) -> materials (friction = sqrt(fa fb), restitution = max) -> velocity
//   integration.
#pragma once
#include "ad_geom.cuh"

#if !defined(__CUDACC__)
#include <algorithm>
#include <cstring>
#endif

namespace pe {
namespace ad {

constexpr uint32_t kAdMaxColors = 128;  // colours per window of the per-body colour masks
constexpr int kDualChunk = 4;
constexpr int kDualInputs = 29;  // xA 3, qA 4, xB 3, qB 4, v1A 3, w1A 3, v1B 3, w1B 3, mA, mB, restitution
constexpr int kTapeScalars = 24; // vA, wA, vB, wB, then 4 x (n, t1, t2)
constexpr int kPmScalars = 20;   // IA (9), IB (9), imA, imB

enum : uint32_t { kAdErrPairs = 1, kAdErrManifolds = 2, kAdErrColors = 4, kAdErrCache = 8, kAdErrReplay = 16 };

// ------------------------------------------------------------------ teams ---
#if !defined(__CUDACC__)
struct HostTeam {
    static uint32_t tid() { return 0; }
    static uint32_t size() { return 1; }
    static void sync() {}
    template <class S> static void add(S *p, S v) { *p += v; }
    static void orErr(uint32_t *p, uint32_t v) { *p |= v; }
    static uint32_t scan(uint32_t v, uint32_t &total) {
        total = v;
        return 0;
    }
    static void sortU64(unsigned long long *k, uint32_t n) { std::sort(k, k + n); }
};
#else
struct BlockTeam {
    static __device__ __forceinline__ uint32_t tid() { return threadIdx.x; }
    static __device__ __forceinline__ uint32_t size() { return blockDim.x; }
    static __device__ __forceinline__ void sync() { __syncthreads(); }
    template <class S> static __device__ __forceinline__ void add(S *p, S v) { atomicAdd(p, v); }
    static __device__ __forceinline__ void orErr(uint32_t *p, uint32_t v) { atomicOr(p, v); }
    // Exclusive scan over the block (multiple of 32 threads, <= 1024).
    static __device__ uint32_t scan(uint32_t v, uint32_t &total) {
        __shared__ uint32_t s[33];
        const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        uint32_t incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t n = __shfl_up_sync(0xffffffffu, incl, o);
            if ((int)lane >= o) incl += n;
        }
        if (lane == 31) s[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            const uint32_t x = lane < nw ? s[lane] : 0u;
            uint32_t xi = x;
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
    // Bitonic sort of n (power of two) keys by the whole block.
    static __device__ void sortU64(unsigned long long *k, uint32_t n) {
        for (uint32_t size = 2; size <= n; size <<= 1)
            for (uint32_t j = size >> 1; j > 0; j >>= 1) {
                for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
                    const uint32_t ixj = i ^ j;
                    if (ixj > i) {
                        const unsigned long long a = k[i], b = k[ixj];
                        const bool up = (i & size) == 0;
                        if ((a > b) == up) {
                            k[i] = b;
                            k[ixj] = a;
                        }
                    }
                }
                __syncthreads();
            }
    }
};
#endif

AD_HD uint32_t nextPow2u(uint32_t v) {
    uint32_t p = 1;
    while (p < v) p <<= 1;
    return p;
}

// Manifold priority for the colouring (a bijective 32-bit mix of the index).
AD_HD uint32_t adColorPriority(uint32_t m) {
    uint32_t h = m;
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

// ------------------------------------------------------------------ views ---
template <class S> struct WorldParams {
    uint32_t n;
    const uint8_t *shape;     // 0 sphere, 1 box
    const uint8_t *isStatic;
    const S *dims;            // radius / half extents, 3 per body
    const S *iinv;            // diagonal local inverse inertia, 3 per body
    const S *mass, *mu, *rest;
    S gx, gy, gz, dt;
    int iterations;
    uint32_t maxPairs, maxManifolds;  // maxManifolds is a power of two
};

template <class S> struct StateView {
    S *x, *q, *v, *w;  // 3, 4, 3, 3 per body
};

// Warm-start cache (sorted by (body A, body B), stable in solve order).
template <class S> struct CacheView {
    uint32_t *count;
    unsigned long long *key;  // body A << 32 | body B
    S *anchorA, *anchorB;     // 3 per entry
    S *lam;                   // normal, tangent 1, tangent 2
    uint32_t cap;
};

template <class S> struct StepScratch {
    S *aabb;                        // 6 per body
    uint32_t *pairA, *pairB;        // maxPairs
    uint32_t *mA, *mB, *mCount;     // manifolds in pair order
    uint32_t *mFeature;             // 4 per manifold
    S *mNormal;                     // 3
    S *mMu, *mRest;
    S *mAnchorA, *mAnchorB;         // 12 each
    S *mDepth;                      // 4
    uint32_t *color, *order;        // maxManifolds
    unsigned long long *sortKeys;   // maxManifolds
    unsigned long long *bodyUsed;   // 2 per body
    uint32_t *colorStart;           // maxManifolds + 1 (colours <= manifolds)
    S *pp;                          // kPreparedScalars per (k, p)
    S *pm;                          // kPmScalars per k
    S *lam;                         // 3 per (k, p)
    S *lamInit;                     // 3 per (k, p)
    int32_t *match;                 // per (k, p): matched cache entry or -1
    S *tape;                        // iterations * maxManifolds * kTapeScalars
    uint32_t *cacheSrc;             // per cache-out entry: k * 4 + p
    uint32_t *counts;               // [0] pairs, [1] manifolds, [2] colours, [3] error bits
    // broadphase scratch (not recorded: it may be shared by the steps of a segment)
    unsigned long long *bpEntries;  // nextPow2(n): (min.x key << 32) | body
    unsigned long long *bpPairs;    // nextPow2(maxPairs): (first << 32) | second
};

// Order-preserving 32-bit key of a float (the sort order of the sweep).
AD_HD uint32_t adOrderedKey(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
AD_HD uint32_t adOrderedKey(double d) { return adOrderedKey((float)d); }

template <class S> struct AdjointView {
    S *ax, *aq, *av, *aw;        // per body (3, 4, 3, 3)
    S *alam;                     // 3 per (k, p)
    S *app;                      // kPreparedScalars per (k, p)
    S *apm;                      // kPmScalars per k
    S *an;                       // 3 per k
    S *amuM, *arestM;            // per k
    S *acache;                   // 3 per entry of the step's input cache
    S *amass, *amu, *arest;      // per body, accumulated over steps
};

template <class S> AD_HD V3<S> ld3(const S *p, uint32_t i) { return {p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }
template <class S> AD_HD void st3(S *p, uint32_t i, const V3<S> &v) {
    p[3 * i] = v.x;
    p[3 * i + 1] = v.y;
    p[3 * i + 2] = v.z;
}
template <class S> AD_HD Q<S> ld4q(const S *p, uint32_t i) { return {p[4 * i], p[4 * i + 1], p[4 * i + 2], p[4 * i + 3]}; }
template <class S> AD_HD void st4q(S *p, uint32_t i, const Q<S> &q) {
    p[4 * i] = q.x;
    p[4 * i + 1] = q.y;
    p[4 * i + 2] = q.z;
    p[4 * i + 3] = q.w;
}
template <class S> AD_HD M3<S> ldm(const S *p) { return {p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], p[8]}; }

// RigidBody::getInverseMass (rigid_body.hpp:74-77)
template <class S> AD_HD S inverseMass(bool isStatic, const S &m) {
    return (isStatic || val(m) <= 0.0f) ? ADL(S, 0.0f) : ADL(S, 1.0f) / m;
}

// ------------------------------------------------------ velocity iterations --
// One contact point of solvePrepared (sequential_impulse_solver.cpp:520-603).
template <class S> struct PointIn {
    V3<S> vA, wA, vB, wB;
    S ln, l1, l2;
};
template <class S>
AD_HDN void pointForward(const V3<S> &n, const S &friction, const S *c, const S &imA, const S &imB, bool sA, bool sB,
                        PointIn<S> &st) {
    const S iem = c[kPIem];
    if (val(iem) <= 0.0f) return;
    const V3<S> offA = pv(c, kPOffA), offB = pv(c, kPOffB), t1 = pv(c, kPT1), t2 = pv(c, kPT2);
    const V3<S> vA = st.vA + cross(st.wA, offA), vB = st.vB + cross(st.wB, offB);
    const V3<S> rel = vB - vA;
    const S vn = dot(rel, n);
    const S delta = -(vn + c[kPRv] - c[kPBias]) / iem;
    const S prev = st.ln;
    st.ln = smax(prev + delta, ADL(S, 0.0f));
    const S applied = st.ln - prev;
    const V3<S> impulse = n * applied;
    if (!sA) {
        st.vA += (-impulse) * imA;
        st.wA += pv(c, kPNrA) * (-applied);
    }
    if (!sB) {
        st.vB += impulse * imB;
        st.wB += pv(c, kPNrB) * applied;
    }
    if (val(c[kPItm00]) <= 0.0f || val(c[kPItm11]) <= 0.0f) return;
    const S limit = smax(friction, ADL(S, 0.0f)) * st.ln;
    const S tv1 = dot(rel, t1) + c[kPNtr1] * applied;
    const S tv2 = dot(rel, t2) + c[kPNtr2] * applied;
    const S d1 = -(c[kPItm00] * tv1 + c[kPItm01] * tv2);
    const S d2 = -(c[kPItm01] * tv1 + c[kPItm11] * tv2);
    const S p1 = st.l1, p2 = st.l2;
    st.l1 = st.l1 + d1;
    st.l2 = st.l2 + d2;
    const S lsq = st.l1 * st.l1 + st.l2 * st.l2;
    if (val(lsq) > val(limit * limit)) {
        const S s = limit / ssqrt(lsq);
        st.l1 = st.l1 * s;
        st.l2 = st.l2 * s;
    }
    const S a1 = st.l1 - p1, a2 = st.l2 - p2;
    const V3<S> ti = t1 * a1 + t2 * a2;
    const V3<S> rA = pv(c, kPTrA1) * a1 + pv(c, kPTrA2) * a2;
    const V3<S> rB = pv(c, kPTrB1) * a1 + pv(c, kPTrB2) * a2;
    if (!sA) {
        st.vA += (-ti) * imA;
        st.wA += -rA;
    }
    if (!sB) {
        st.vB += ti * imB;
        st.wB += rB;
    }
}

// Reverse of pointForward.  `in` holds the point's inputs; `a` holds the
// adjoints of its outputs on entry and of its inputs on exit.  Adjoints of the
// prepared constants go to ac[], of the normal to an, of the friction to amu,
// of the inverse masses to aimA / aimB.
template <class S>
AD_HDN void pointReverse(const V3<S> &n, const S &friction, const S *c, const S &imA, const S &imB, bool sA, bool sB,
                        const PointIn<S> &in, PointIn<S> &a, S *ac, V3<S> &an, S &amu, S &aimA, S &aimB) {
    const S iem = c[kPIem];
    if (val(iem) <= 0.0f) return;
    const S z = S(0);
    const V3<S> offA = pv(c, kPOffA), offB = pv(c, kPOffB), t1 = pv(c, kPT1), t2 = pv(c, kPT2);
    // recompute the forward intermediates
    const V3<S> vAp = in.vA + cross(in.wA, offA), vBp = in.vB + cross(in.wB, offB);
    const V3<S> rel = vBp - vAp;
    const S vn = dot(rel, n);
    const S num = vn + c[kPRv] - c[kPBias];
    const S delta = -num / iem;
    const S prev = in.ln;
    const S raw = prev + delta;
    const S ln = smax(raw, z);
    const S applied = ln - prev;
    const V3<S> impulse = n * applied;
    S aln = a.ln, aapplied = z, aprev = z;
    V3<S> arel{z, z, z};
    const bool fric = !(c[kPItm00] <= z || c[kPItm11] <= z);
    if (fric) {
        const S mu0 = smax(friction, z);
        const S limit = mu0 * ln;
        const S tv1 = dot(rel, t1) + c[kPNtr1] * applied;
        const S tv2 = dot(rel, t2) + c[kPNtr2] * applied;
        const S d1 = -(c[kPItm00] * tv1 + c[kPItm01] * tv2);
        const S d2 = -(c[kPItm01] * tv1 + c[kPItm11] * tv2);
        const S p1 = in.l1, p2 = in.l2;
        const S r1 = p1 + d1, r2 = p2 + d2;
        const S lsq = r1 * r1 + r2 * r2;
        const bool scaled = lsq > limit * limit;
        S f1 = r1, f2 = r2, L = z;
        if (scaled) {
            L = ssqrt(lsq);
            const S s = limit / L;
            f1 = r1 * s;
            f2 = r2 * s;
        }
        const S a1 = f1 - p1, a2 = f2 - p2;
        const V3<S> ti = t1 * a1 + t2 * a2;
        // velocities after the friction update
        V3<S> ati{z, z, z}, arA{z, z, z}, arB{z, z, z};
        if (!sB) {
            ati += a.vB * imB;
            aimB = aimB + dot(a.vB, ti);
            arB = a.wB;
        }
        if (!sA) {
            ati += -(a.vA * imA);
            aimA = aimA - dot(a.vA, ti);
            arA = -a.wA;
        }
        S aa1 = dot(ati, t1) + dot(arA, pv(c, kPTrA1)) + dot(arB, pv(c, kPTrB1));
        S aa2 = dot(ati, t2) + dot(arA, pv(c, kPTrA2)) + dot(arB, pv(c, kPTrB2));
        auto acc3 = [&](int f, const V3<S> &v) {
            ac[3 * f] = ac[3 * f] + v.x;
            ac[3 * f + 1] = ac[3 * f + 1] + v.y;
            ac[3 * f + 2] = ac[3 * f + 2] + v.z;
        };
        acc3(kPT1, ati * a1);
        acc3(kPT2, ati * a2);
        acc3(kPTrA1, arA * a1);
        acc3(kPTrA2, arA * a2);
        acc3(kPTrB1, arB * a1);
        acc3(kPTrB2, arB * a2);
        // a = f - p; the outputs l1, l2 are f
        S af1 = a.l1 + aa1, af2 = a.l2 + aa2;
        S ap1 = -aa1, ap2 = -aa2;
        S ar1 = af1, ar2 = af2, alimit = z;
        if (scaled) {
            const S u1 = r1 / L, u2 = r2 / L;
            const S ua = u1 * af1 + u2 * af2;
            const S k = limit / L;
            ar1 = k * (af1 - u1 * ua);
            ar2 = k * (af2 - u2 * ua);
            alimit = ua;
        }
        ap1 = ap1 + ar1;
        ap2 = ap2 + ar2;
        const S ad1 = ar1, ad2 = ar2;
        const S atv1 = -(ad1 * c[kPItm00] + ad2 * c[kPItm01]);
        const S atv2 = -(ad1 * c[kPItm01] + ad2 * c[kPItm11]);
        ac[kPItm00] = ac[kPItm00] - ad1 * tv1;
        ac[kPItm01] = ac[kPItm01] - (ad1 * tv2 + ad2 * tv1);
        ac[kPItm11] = ac[kPItm11] - ad2 * tv2;
        arel += t1 * atv1 + t2 * atv2;
        acc3(kPT1, rel * atv1);
        acc3(kPT2, rel * atv2);
        ac[kPNtr1] = ac[kPNtr1] + atv1 * applied;
        ac[kPNtr2] = ac[kPNtr2] + atv2 * applied;
        aapplied = aapplied + atv1 * c[kPNtr1] + atv2 * c[kPNtr2];
        if (!(friction < z)) amu = amu + alimit * ln;
        aln = aln + alimit * mu0;
        a.l1 = ap1;
        a.l2 = ap2;
    }
    // normal update
    V3<S> aimp{z, z, z};
    if (!sB) {
        aimp += a.vB * imB;
        aimB = aimB + dot(a.vB, impulse);
        const V3<S> nrB = pv(c, kPNrB);
        ac[3 * kPNrB] = ac[3 * kPNrB] + a.wB.x * applied;
        ac[3 * kPNrB + 1] = ac[3 * kPNrB + 1] + a.wB.y * applied;
        ac[3 * kPNrB + 2] = ac[3 * kPNrB + 2] + a.wB.z * applied;
        aapplied = aapplied + dot(a.wB, nrB);
    }
    if (!sA) {
        aimp += -(a.vA * imA);
        aimA = aimA - dot(a.vA, impulse);
        const V3<S> nrA = pv(c, kPNrA);
        ac[3 * kPNrA] = ac[3 * kPNrA] - a.wA.x * applied;
        ac[3 * kPNrA + 1] = ac[3 * kPNrA + 1] - a.wA.y * applied;
        ac[3 * kPNrA + 2] = ac[3 * kPNrA + 2] - a.wA.z * applied;
        aapplied = aapplied - dot(a.wA, nrA);
    }
    an += aimp * applied;
    aapplied = aapplied + dot(aimp, n);
    aln = aln + aapplied;
    aprev = aprev - aapplied;
    const S araw = (raw < z) ? z : aln;
    aprev = aprev + araw;
    const S adelta = araw;
    const S anum = -adelta / iem;
    ac[kPIem] = ac[kPIem] + adelta * num / (iem * iem);
    ac[kPRv] = ac[kPRv] + anum;
    ac[kPBias] = ac[kPBias] - anum;
    arel += n * anum;
    an += rel * anum;
    // rel = (vB + wB x offB) - (vA + wA x offA)
    a.vB += arel;
    a.vA += -arel;
    V3<S> aoffB{z, z, z}, aoffA{z, z, z}, awB = a.wB, awA = a.wA;
    crossAdj(in.wB, offB, arel, awB, aoffB);
    crossAdj(in.wA, offA, -arel, awA, aoffA);
    a.wB = awB;
    a.wA = awA;
    ac[3 * kPOffB] = ac[3 * kPOffB] + aoffB.x;
    ac[3 * kPOffB + 1] = ac[3 * kPOffB + 1] + aoffB.y;
    ac[3 * kPOffB + 2] = ac[3 * kPOffB + 2] + aoffB.z;
    ac[3 * kPOffA] = ac[3 * kPOffA] + aoffA.x;
    ac[3 * kPOffA + 1] = ac[3 * kPOffA + 1] + aoffA.y;
    ac[3 * kPOffA + 2] = ac[3 * kPOffA + 2] + aoffA.z;
    a.ln = aprev;
}

// ------------------------------------------------------------------ forward --
template <class S, class T>
AD_HD void forwardStep(const WorldParams<S> &W, const StateView<S> &in, const CacheView<S> &cin, StateView<S> out,
                       CacheView<S> cout, StepScratch<S> sc, bool record) {
    const uint32_t tid = T::tid(), nt = T::size(), n = W.n;
    const S z = ADL(S, 0.0f);
    const V3<S> g{W.gx, W.gy, W.gz};
    // 1. velocity integration (RigidBody::integrateVelocity, no applied force) and AABBs
    for (uint32_t i = tid; i < n; i += nt) {
        V3<S> v = ld3(in.v, i);
        const bool st = W.isStatic[i] != 0;
        if (!st) {
            const V3<S> f{z, z, z};
            const V3<S> acc = g + f * inverseMass(false, W.mass[i]);
            v += acc * W.dt;
        }
        st3(out.v, i, v);
        st3(out.w, i, ld3(in.w, i));
        const V3<S> p = ld3(in.x, i);
        const Q<S> q = ld4q(in.q, i);
        V3<S> mn, mx;
        if (W.shape[i] == 0) {
            const S r = W.dims[3 * i];
            const V3<S> rr{r, r, r};
            mn = p - rr;
            mx = p + rr;
        } else {
            const M3<S> m = toMat3(q);
            const S hx = W.dims[3 * i], hy = W.dims[3 * i + 1], hz = W.dims[3 * i + 2];
            const V3<S> e{sabs(m.m00) * hx + sabs(m.m01) * hy + sabs(m.m02) * hz,
                          sabs(m.m10) * hx + sabs(m.m11) * hy + sabs(m.m12) * hz,
                          sabs(m.m20) * hx + sabs(m.m21) * hy + sabs(m.m22) * hz};
            mn = p - e;
            mx = p + e;
        }
        st3(sc.aabb, 2 * i, mn);
        st3(sc.aabb, 2 * i + 1, mx);
    }
    if (tid == 0) {
        sc.counts[0] = 0;
        sc.counts[1] = 0;
        sc.counts[3] = 0;
    }
    T::sync();
    // 2. every pair (i < j) with overlapping AABBs (touching counts), in
    // lexicographic order: sort and sweep along x (broadphase.cpp:195-291) —
    // bodies sorted by min.x, each tested against the later ones whose min.x
    // does not exceed its max.x (the one of an overlapping pair sorted first
    // always meets the other) — then the pairs sorted by (first, second).
    const uint32_t n2 = nextPow2u(n > 0 ? n : 1);
    for (uint32_t i = tid; i < n2; i += nt)
        sc.bpEntries[i] = i < n ? ((unsigned long long)adOrderedKey(val(sc.aabb[6 * i])) << 32) | i : ~0ull;
    T::sync();
    T::sortU64(sc.bpEntries, n2);
    T::sync();
    auto overlapsYZ = [&](uint32_t a, uint32_t b) {
        const V3<S> amn = ld3(sc.aabb, 2 * a), amx = ld3(sc.aabb, 2 * a + 1);
        const V3<S> bmn = ld3(sc.aabb, 2 * b), bmx = ld3(sc.aabb, 2 * b + 1);
        return val(amn.y) <= val(bmx.y) && val(amx.y) >= val(bmn.y) && val(amn.z) <= val(bmx.z) &&
               val(amx.z) >= val(bmn.z);
    };
    uint32_t P = 0;
    for (uint32_t k0 = 0; k0 < n; k0 += nt) {
        const uint32_t k = k0 + tid;
        uint32_t hits = 0;
        uint32_t i = 0;
        if (k < n) {
            i = (uint32_t)sc.bpEntries[k];
            const auto maxX = val(sc.aabb[6 * i + 3]);
            for (uint32_t kk = k + 1; kk < n; ++kk) {
                const uint32_t j = (uint32_t)sc.bpEntries[kk];
                if (val(sc.aabb[6 * j]) > maxX) break;
                if (overlapsYZ(i, j)) ++hits;
            }
        }
        uint32_t cnt;
        uint32_t slot = P + T::scan(hits, cnt);
        if (k < n && hits) {
            const auto maxX = val(sc.aabb[6 * i + 3]);
            for (uint32_t kk = k + 1; kk < n; ++kk) {
                const uint32_t j = (uint32_t)sc.bpEntries[kk];
                if (val(sc.aabb[6 * j]) > maxX) break;
                if (!overlapsYZ(i, j)) continue;
                if (slot < W.maxPairs)
                    sc.bpPairs[slot] = ((unsigned long long)(i < j ? i : j) << 32) | (i < j ? j : i);
                ++slot;
            }
        }
        P += cnt;
    }
    if (P > W.maxPairs) {
        if (tid == 0) T::orErr(&sc.counts[3], kAdErrPairs);
        P = W.maxPairs;
    }
    const uint32_t P2 = nextPow2u(P > 0 ? P : 1);
    for (uint32_t p = P + tid; p < P2; p += nt) sc.bpPairs[p] = ~0ull;
    T::sync();
    T::sortU64(sc.bpPairs, P2);
    T::sync();
    for (uint32_t p = tid; p < P; p += nt) {
        sc.pairA[p] = (uint32_t)(sc.bpPairs[p] >> 32);
        sc.pairB[p] = (uint32_t)sc.bpPairs[p];
    }
    if (tid == 0) sc.counts[0] = P;
    T::sync();
    // 3. narrowphase in pair order, manifolds compacted in that order
    uint32_t M = 0;
    for (uint32_t t0 = 0; t0 < P; t0 += nt) {
        const uint32_t p = t0 + tid;
        Contact<S> c;
        c.count = 0;
        bool hit = false;
        uint32_t a = 0, b = 0;
        if (p < P) {
            a = sc.pairA[p];
            b = sc.pairB[p];
            const Tf<S> tA{ld3(in.x, a), ld4q(in.q, a)}, tB{ld3(in.x, b), ld4q(in.q, b)};
            hit = contactPair<S>(W.shape[a], ld3(W.dims, a), tA, W.shape[b], ld3(W.dims, b), tB, c);
        }
        uint32_t cnt;
        const uint32_t m = M + T::scan(hit ? 1u : 0u, cnt);
        if (hit && m < W.maxManifolds) {
            sc.mA[m] = a;
            sc.mB[m] = b;
            sc.mCount[m] = c.count;
            st3(sc.mNormal, m, c.normal);
            sc.mRest[m] = smax(W.rest[a], W.rest[b]);
            sc.mMu[m] = ssqrt(smax(W.mu[a], z) * smax(W.mu[b], z));
            for (uint32_t k = 0; k < 4; ++k) {
                const bool live = k < c.count;
                st3(sc.mAnchorA, 4 * m + k, live ? c.anchorA[k] : V3<S>{z, z, z});
                st3(sc.mAnchorB, 4 * m + k, live ? c.anchorB[k] : V3<S>{z, z, z});
                sc.mDepth[4 * m + k] = live ? c.depth[k] : z;
                sc.mFeature[4 * m + k] = live ? c.feature[k] : 0u;
            }
        }
        M += cnt;
    }
    if (M > W.maxManifolds) {
        if (tid == 0) T::orErr(&sc.counts[3], kAdErrManifolds);
        M = W.maxManifolds;
    }
    if (tid == 0) sc.counts[1] = M;
    // 4. colouring: greedy in decreasing priority over manifolds that share a
    // dynamic body (the engine's colouring), then order = (colour, index)
    const uint32_t M2 = nextPow2u(M > 0 ? M : 1);
    for (uint32_t i = tid; i < M2; i += nt)
        sc.sortKeys[i] = i < M ? ((unsigned long long)(~adColorPriority(i)) << 32) | i : ~0ull;
    for (uint32_t i = tid; i < 2 * n; i += nt) sc.bodyUsed[i] = 0ull;
    T::sync();
    T::sortU64(sc.sortKeys, M2);
    T::sync();
    if (tid == 0) {
        // Colour windows of kAdMaxColors: a manifold whose higher-priority
        // neighbours use the whole window waits for the next window, in which
        // only the waiting manifolds take colours (the engine's rule, so the
        // same colouring); no colour limit.
        constexpr uint32_t kWaiting = 0xFFFFFFFFu;
        for (uint32_t r = 0; r < M; ++r) sc.color[(uint32_t)sc.sortKeys[r]] = kWaiting;
        uint32_t colors = 0, base = 0, waiting = M;
        while (waiting) {
            uint32_t deferred = 0;
            for (uint32_t r = 0; r < M; ++r) {
                const uint32_t m = (uint32_t)sc.sortKeys[r];
                if (sc.color[m] != kWaiting) continue;
                const uint32_t a = sc.mA[m], b = sc.mB[m];
                const bool da = !W.isStatic[a], db = !W.isStatic[b];
                unsigned long long u0 = 0, u1 = 0;
                if (da) {
                    u0 |= sc.bodyUsed[2 * a];
                    u1 |= sc.bodyUsed[2 * a + 1];
                }
                if (db) {
                    u0 |= sc.bodyUsed[2 * b];
                    u1 |= sc.bodyUsed[2 * b + 1];
                }
                uint32_t local = kAdMaxColors;
                for (uint32_t k = 0; k < kAdMaxColors && local == kAdMaxColors; ++k) {
                    const unsigned long long w = k < 64 ? u0 : u1;
                    if (!((w >> (k & 63)) & 1ull)) local = k;
                }
                if (local == kAdMaxColors) {
                    ++deferred;
                    continue;
                }
                const uint32_t c = base + local;
                sc.color[m] = c;
                const unsigned long long bit = 1ull << (local & 63);
                if (da) sc.bodyUsed[2 * a + (local >> 6)] |= bit;
                if (db) sc.bodyUsed[2 * b + (local >> 6)] |= bit;
                if (c + 1 > colors) colors = c + 1;
            }
            waiting = deferred;
            if (waiting) {
                base += kAdMaxColors;
                for (uint32_t i = 0; i < 2 * n; ++i) sc.bodyUsed[i] = 0ull;
            }
        }
        sc.counts[2] = colors;
    }
    T::sync();
    for (uint32_t i = tid; i < M2; i += nt)
        sc.sortKeys[i] = i < M ? ((unsigned long long)sc.color[i] << 32) | i : ~0ull;
    T::sync();
    T::sortU64(sc.sortKeys, M2);
    T::sync();
    const uint32_t C = sc.counts[2];
    for (uint32_t k = tid; k < M; k += nt) {
        sc.order[k] = (uint32_t)sc.sortKeys[k];
        const uint32_t ck = (uint32_t)(sc.sortKeys[k] >> 32);
        const uint32_t cp = k == 0 ? 0xFFFFFFFFu : (uint32_t)(sc.sortKeys[k - 1] >> 32);
        for (uint32_t c = (k == 0 ? 0 : cp + 1); c <= ck; ++c) sc.colorStart[c] = k;
    }
    if (tid == 0) sc.colorStart[C] = M;
    T::sync();
    // 5. prepare + warm-start matching (sequential_impulse_solver.cpp:101-214, :448-490)
    const S inverseDt = ADL(S, 1.0f) / smax(W.dt, ADL(S, 1e-6f));
    const uint32_t cacheN = *cin.count;
    for (uint32_t k = tid; k < M; k += nt) {
        const uint32_t m = sc.order[k];
        const uint32_t a = sc.mA[m], b = sc.mB[m];
        const bool sA = W.isStatic[a] != 0, sB = W.isStatic[b] != 0;
        const Q<S> qA = ld4q(in.q, a), qB = ld4q(in.q, b);
        const M3<S> IA = inverseInertiaWorld(qA, W.iinv[3 * a], W.iinv[3 * a + 1], W.iinv[3 * a + 2]);
        const M3<S> IB = inverseInertiaWorld(qB, W.iinv[3 * b], W.iinv[3 * b + 1], W.iinv[3 * b + 2]);
        const S imA = inverseMass(sA, W.mass[a]), imB = inverseMass(sB, W.mass[b]);
        S *pm = sc.pm + (size_t)k * kPmScalars;
        const S *ia = &IA.m00, *ib = &IB.m00;
        for (int e = 0; e < 9; ++e) {
            pm[e] = ia[e];
            pm[9 + e] = ib[e];
        }
        pm[18] = imA;
        pm[19] = imB;
        const V3<S> n3 = ld3(sc.mNormal, m);
        const V3<S> linA = ld3(out.v, a), angA = ld3(out.w, a), linB = ld3(out.v, b), angB = ld3(out.w, b);
        const unsigned long long key = ((unsigned long long)a << 32) | b;
        uint32_t lo = 0, hi = cacheN;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (cin.key[mid] < key) lo = mid + 1;
            else hi = mid;
        }
        uint32_t re = lo;
        while (re < cacheN && cin.key[re] == key) ++re;
        const S friction = sc.mMu[m];
        const uint32_t npts = sc.mCount[m];
        for (uint32_t p = 0; p < 4; ++p) {
            const size_t kp = (size_t)k * 4 + p;
            S *pp = sc.pp + kp * kPreparedScalars;
            for (int e = 0; e < kPreparedScalars; ++e) pp[e] = z;
            S l0 = z, l1 = z, l2 = z;
            int32_t match = -1;
            if (p < npts) {
                const V3<S> anA = ld3(sc.mAnchorA, 4 * m + p), anB = ld3(sc.mAnchorB, 4 * m + p);
                Prepared<S> pr;
                preparePoint(n3, anA, anB, sc.mDepth[4 * m + p], qA, qB, IA, IB, imA, imB, linA, angA, linB, angB,
                             sc.mRest[m], inverseDt, pr);
                preparedPack(pr, pp);
                if (pr.tangentValid && !(val(pr.iem) <= 0.0f)) {
                    const float matchSq = 0.05f * 0.05f;
                    for (uint32_t e = lo; e < re; ++e) {
                        const V3<S> da = ld3(cin.anchorA, e) - anA, db = ld3(cin.anchorB, e) - anB;
                        if (val(dot(da, da)) > matchSq || val(dot(db, db)) > matchSq) continue;
                        const S cn = cin.lam[3 * e], c1 = cin.lam[3 * e + 1], c2 = cin.lam[3 * e + 2];
                        const S ni = smax(cn, z);
                        const S limit = smax(friction, z) * ni;
                        const S tlsq = c1 * c1 + c2 * c2;
                        const S scale = val(tlsq) > val(limit * limit) ? limit / ssqrt(tlsq) : ADL(S, 1.0f);
                        l0 = ni;
                        l1 = c1 * scale;
                        l2 = c2 * scale;
                        match = (int32_t)e;
                        break;
                    }
                }
            }
            sc.match[kp] = match;
            sc.lamInit[3 * kp] = sc.lam[3 * kp] = l0;
            sc.lamInit[3 * kp + 1] = sc.lam[3 * kp + 1] = l1;
            sc.lamInit[3 * kp + 2] = sc.lam[3 * kp + 2] = l2;
        }
    }
    T::sync();
    // 6. warm start, colour by colour (warmStartPrepared :453-490)
    for (uint32_t c = 0; c < C; ++c) {
        for (uint32_t k = sc.colorStart[c] + tid; k < sc.colorStart[c + 1]; k += nt) {
            const uint32_t m = sc.order[k];
            const uint32_t a = sc.mA[m], b = sc.mB[m];
            const bool sA = W.isStatic[a] != 0, sB = W.isStatic[b] != 0;
            const S *pm = sc.pm + (size_t)k * kPmScalars;
            const M3<S> IA = ldm(pm), IB = ldm(pm + 9);
            const V3<S> n3 = ld3(sc.mNormal, m);
            V3<S> linA = ld3(out.v, a), angA = ld3(out.w, a), linB = ld3(out.v, b), angB = ld3(out.w, b);
            bool any = false;
            for (uint32_t p = 0; p < sc.mCount[m]; ++p) {
                const size_t kp = (size_t)k * 4 + p;
                if (sc.match[kp] < 0) continue;
                const S *pp = sc.pp + kp * kPreparedScalars;
                const V3<S> wi = n3 * sc.lamInit[3 * kp] + pv(pp, kPT1) * sc.lamInit[3 * kp + 1] +
                                 pv(pp, kPT2) * sc.lamInit[3 * kp + 2];
                const V3<S> nw = -wi;
                if (!sA) {
                    linA += nw * pm[18];
                    angA += mul(IA, cross(pv(pp, kPOffA), nw));
                }
                if (!sB) {
                    linB += wi * pm[19];
                    angB += mul(IB, cross(pv(pp, kPOffB), wi));
                }
                any = true;
            }
            if (!any) continue;
            if (!sA) {
                st3(out.v, a, linA);
                st3(out.w, a, angA);
            }
            if (!sB) {
                st3(out.v, b, linB);
                st3(out.w, b, angB);
            }
        }
        T::sync();
    }
    // 7. velocity iterations in colour order, with the tape of each manifold update
    for (int it = 0; it < W.iterations; ++it)
        for (uint32_t c = 0; c < C; ++c) {
            for (uint32_t k = sc.colorStart[c] + tid; k < sc.colorStart[c + 1]; k += nt) {
                const uint32_t m = sc.order[k];
                const uint32_t a = sc.mA[m], b = sc.mB[m];
                const bool sA = W.isStatic[a] != 0, sB = W.isStatic[b] != 0;
                const S *pm = sc.pm + (size_t)k * kPmScalars;
                const V3<S> n3 = ld3(sc.mNormal, m);
                PointIn<S> s{ld3(out.v, a), ld3(out.w, a), ld3(out.v, b), ld3(out.w, b), z, z, z};
                if (record) {
                    S *tp = sc.tape + ((size_t)it * W.maxManifolds + k) * kTapeScalars;
                    st3(tp, 0, s.vA);
                    st3(tp, 1, s.wA);
                    st3(tp, 2, s.vB);
                    st3(tp, 3, s.wB);
                    for (int e = 0; e < 12; ++e) tp[12 + e] = sc.lam[(size_t)k * 12 + e];
                }
                for (uint32_t p = 0; p < sc.mCount[m]; ++p) {
                    const size_t kp = (size_t)k * 4 + p;
                    s.ln = sc.lam[3 * kp];
                    s.l1 = sc.lam[3 * kp + 1];
                    s.l2 = sc.lam[3 * kp + 2];
                    pointForward(n3, sc.mMu[m], sc.pp + kp * kPreparedScalars, pm[18], pm[19], sA, sB, s);
                    sc.lam[3 * kp] = s.ln;
                    sc.lam[3 * kp + 1] = s.l1;
                    sc.lam[3 * kp + 2] = s.l2;
                }
                if (!sA) {
                    st3(out.v, a, s.vA);
                    st3(out.w, a, s.wA);
                }
                if (!sB) {
                    st3(out.v, b, s.vB);
                    st3(out.w, b, s.wB);
                }
            }
            T::sync();
        }
    // 8. cache rebuild: entries sorted by (body A, body B), stable in solve order (:623-681)
    for (uint32_t i = tid; i < M2; i += nt) {
        unsigned long long key = ~0ull;
        if (i < M) {
            const uint32_t m = sc.order[i];
            key = ((unsigned long long)sc.mA[m] << 44) | ((unsigned long long)sc.mB[m] << 24) | i;
        }
        sc.sortKeys[i] = key;
    }
    T::sync();
    T::sortU64(sc.sortKeys, M2);
    T::sync();
    if (tid == 0) {
        uint32_t e = 0;
        for (uint32_t r = 0; r < M; ++r) {
            const uint32_t k = (uint32_t)(sc.sortKeys[r] & 0xFFFFFFu);
            const uint32_t m = sc.order[k];
            for (uint32_t p = 0; p < sc.mCount[m]; ++p, ++e) {
                if (e >= cout.cap) {
                    sc.counts[3] |= kAdErrCache;
                    break;
                }
                const size_t kp = (size_t)k * 4 + p;
                cout.key[e] = ((unsigned long long)sc.mA[m] << 32) | sc.mB[m];
                st3(cout.anchorA, e, ld3(sc.mAnchorA, 4 * m + p));
                st3(cout.anchorB, e, ld3(sc.mAnchorB, 4 * m + p));
                cout.lam[3 * e] = sc.lam[3 * kp];
                cout.lam[3 * e + 1] = sc.lam[3 * kp + 1];
                cout.lam[3 * e + 2] = sc.lam[3 * kp + 2];
                sc.cacheSrc[e] = (uint32_t)kp;
            }
        }
        *cout.count = e < cout.cap ? e : cout.cap;
    }
    // 9. pose integration (rigid_body.cpp:103-125)
    for (uint32_t i = tid; i < n; i += nt) {
        V3<S> pos = ld3(in.x, i);
        Q<S> rot = ld4q(in.q, i);
        if (!W.isStatic[i]) {
            const V3<S> lin = ld3(out.v, i), ang = ld3(out.w, i);
            pos += lin * W.dt;
            const Q<S> spin{ang.x, ang.y, ang.z, z};
            const Q<S> d = qmul(spin, rot);
            const S h = ADL(S, 0.5f) * W.dt;
            rot.x = rot.x + h * d.x;
            rot.y = rot.y + h * d.y;
            rot.z = rot.z + h * d.z;
            rot.w = rot.w + h * d.w;
            rot = qnormalized(rot);
        }
        st3(out.x, i, pos);
        st4q(out.q, i, rot);
    }
    T::sync();
}

// ------------------------------------------------------------------ reverse --
// Contact geometry + preparation of manifold k as a function of the 29 inputs,
// evaluated in dual numbers for directions [base, base + kDualChunk); returns
// the directional derivatives of sum(adjoint * output) in g[].
template <class S>
AD_HDN bool manifoldDualChunk(const WorldParams<S> &W, const StateView<S> &in, const StateView<S> &v1,
                             const StepScratch<S> &sc, const AdjointView<S> &adj, uint32_t k, int base, S *g) {
    using D = Dual<S, kDualChunk>;
    const uint32_t m = sc.order[k];
    const uint32_t a = sc.mA[m], b = sc.mB[m];
    const bool sA = W.isStatic[a] != 0, sB = W.isStatic[b] != 0;
    auto seed = [&](S value, int dir) {
        D r = dconst<S, kDualChunk>(value);
        const int j = dir - base;
        if (j >= 0 && j < kDualChunk) r.d[j] = S(1);
        return r;
    };
    auto seed3 = [&](const S *p, uint32_t i, int dir) {
        return V3<D>{seed(p[3 * i], dir), seed(p[3 * i + 1], dir + 1), seed(p[3 * i + 2], dir + 2)};
    };
    auto c3 = [&](const S *p, uint32_t i) {
        return V3<D>{dconst<S, kDualChunk>(p[3 * i]), dconst<S, kDualChunk>(p[3 * i + 1]),
                     dconst<S, kDualChunk>(p[3 * i + 2])};
    };
    const V3<D> xA = seed3(in.x, a, 0), xB = seed3(in.x, b, 7);
    const Q<D> qA{seed(in.q[4 * a], 3), seed(in.q[4 * a + 1], 4), seed(in.q[4 * a + 2], 5), seed(in.q[4 * a + 3], 6)};
    const Q<D> qB{seed(in.q[4 * b], 10), seed(in.q[4 * b + 1], 11), seed(in.q[4 * b + 2], 12),
                  seed(in.q[4 * b + 3], 13)};
    const V3<D> linA = seed3(v1.v, a, 14), angA = seed3(v1.w, a, 17), linB = seed3(v1.v, b, 20),
                angB = seed3(v1.w, b, 23);
    const D mA = seed(W.mass[a], 26), mB = seed(W.mass[b], 27), rest = seed(sc.mRest[m], 28);
    Contact<D> c;
    const bool hit = contactPair<D>(W.shape[a], c3(W.dims, a), Tf<D>{xA, qA}, W.shape[b], c3(W.dims, b),
                                    Tf<D>{xB, qB}, c);
    bool ok = hit && c.count == sc.mCount[m];
    for (uint32_t p = 0; ok && p < c.count; ++p) ok = c.feature[p] == sc.mFeature[4 * m + p];
    if (!ok) return false;
    const M3<D> IA = inverseInertiaWorld(qA, dconst<S, kDualChunk>(W.iinv[3 * a]),
                                         dconst<S, kDualChunk>(W.iinv[3 * a + 1]),
                                         dconst<S, kDualChunk>(W.iinv[3 * a + 2]));
    const M3<D> IB = inverseInertiaWorld(qB, dconst<S, kDualChunk>(W.iinv[3 * b]),
                                         dconst<S, kDualChunk>(W.iinv[3 * b + 1]),
                                         dconst<S, kDualChunk>(W.iinv[3 * b + 2]));
    const D imA = inverseMass(sA, mA), imB = inverseMass(sB, mB);
    const D inverseDt = ADL(D, 1.0f) / smax(dconst<S, kDualChunk>(W.dt), ADL(D, 1e-6f));
    for (int j = 0; j < kDualChunk; ++j) g[j] = S(0);
    auto acc = [&](const D &o, S adjv) {
        for (int j = 0; j < kDualChunk; ++j) g[j] = g[j] + adjv * o.d[j];
    };
    const S *apm = adj.apm + (size_t)k * kPmScalars;
    const D *ia = &IA.m00, *ib = &IB.m00;
    for (int e = 0; e < 9; ++e) {
        acc(ia[e], apm[e]);
        acc(ib[e], apm[9 + e]);
    }
    acc(imA, apm[18]);
    acc(imB, apm[19]);
    acc(c.normal.x, adj.an[3 * k]);
    acc(c.normal.y, adj.an[3 * k + 1]);
    acc(c.normal.z, adj.an[3 * k + 2]);
    for (uint32_t p = 0; p < c.count; ++p) {
        Prepared<D> pr;
        preparePoint(c.normal, c.anchorA[p], c.anchorB[p], c.depth[p], qA, qB, IA, IB, imA, imB, linA, angA, linB,
                     angB, rest, inverseDt, pr);
        D flat[kPreparedScalars];
        preparedPack(pr, flat);
        const S *ac = adj.app + ((size_t)k * 4 + p) * kPreparedScalars;
        for (int e = 0; e < kPreparedScalars; ++e) acc(flat[e], ac[e]);
    }
    return true;
}

template <class S, class T>
AD_HD void backwardStep(const WorldParams<S> &W, const StateView<S> &in, const CacheView<S> &cin,
                        const StateView<S> &out, StateView<S> v1, const StepScratch<S> &sc, AdjointView<S> adj) {
    const uint32_t tid = T::tid(), nt = T::size(), n = W.n;
    const S z = S(0);
    const uint32_t M = sc.counts[1], C = sc.counts[2];
    // clear the per-step adjoints of constants
    for (uint32_t i = tid; i < M * 4 * kPreparedScalars; i += nt) adj.app[i] = z;
    for (uint32_t i = tid; i < M * kPmScalars; i += nt) adj.apm[i] = z;
    for (uint32_t i = tid; i < 3 * M; i += nt) adj.an[i] = z;
    for (uint32_t i = tid; i < M; i += nt) adj.amuM[i] = adj.arestM[i] = z;
    for (uint32_t i = tid; i < 3 * (*cin.count); i += nt) adj.acache[i] = z;
    // velocities after gravity (the prepare step's input), for the dual pass
    const V3<S> g{W.gx, W.gy, W.gz};
    for (uint32_t i = tid; i < n; i += nt) {
        V3<S> v = ld3(in.v, i);
        if (!W.isStatic[i]) {
            const V3<S> f{z, z, z};
            const V3<S> acc = g + f * inverseMass(false, W.mass[i]);
            v += acc * W.dt;
        }
        st3(v1.v, i, v);
        st3(v1.w, i, ld3(in.w, i));
    }
    // 1. pose integration
    for (uint32_t i = tid; i < n; i += nt) {
        if (W.isStatic[i]) continue;
        const V3<S> ax1 = ld3(adj.ax, i);
        const Q<S> aq1 = ld4q(adj.aq, i);
        V3<S> av = ld3(adj.av, i), aw = ld3(adj.aw, i);
        av += ax1 * W.dt;
        const Q<S> rot = ld4q(in.q, i);
        const V3<S> ang = ld3(out.w, i);
        const Q<S> spin{ang.x, ang.y, ang.z, z};
        const Q<S> d = qmul(spin, rot);
        const S h = S(0.5f) * W.dt;
        const Q<S> u{rot.x + h * d.x, rot.y + h * d.y, rot.z + h * d.z, rot.w + h * d.w};
        const S len = ssqrt(u.x * u.x + u.y * u.y + u.z * u.z + u.w * u.w);
        Q<S> au{z, z, z, z};
        if (len != z) {
            const Q<S> q1{u.x / len, u.y / len, u.z / len, u.w / len};
            const S qa = q1.x * aq1.x + q1.y * aq1.y + q1.z * aq1.z + q1.w * aq1.w;
            au = Q<S>{(aq1.x - q1.x * qa) / len, (aq1.y - q1.y * qa) / len, (aq1.z - q1.z * qa) / len,
                      (aq1.w - q1.w * qa) / len};
        }
        Q<S> arot = au, aspin{z, z, z, z};
        const Q<S> ad{h * au.x, h * au.y, h * au.z, h * au.w};
        qmulAdj(spin, rot, ad, aspin, arot);
        aw += V3<S>{aspin.x, aspin.y, aspin.z};
        st3(adj.av, i, av);
        st3(adj.aw, i, aw);
        st4q(adj.aq, i, arot);
    }
    T::sync();
    // 2. velocity iterations in reverse
    for (int it = W.iterations - 1; it >= 0; --it)
        for (int ci = (int)C - 1; ci >= 0; --ci) {
            const uint32_t c = (uint32_t)ci;
            for (uint32_t k = sc.colorStart[c] + tid; k < sc.colorStart[c + 1]; k += nt) {
                const uint32_t m = sc.order[k];
                const uint32_t a = sc.mA[m], b = sc.mB[m];
                const bool sA = W.isStatic[a] != 0, sB = W.isStatic[b] != 0;
                const S *pm = sc.pm + (size_t)k * kPmScalars;
                const V3<S> n3 = ld3(sc.mNormal, m);
                const S mu = sc.mMu[m];
                const S *tp = sc.tape + ((size_t)it * W.maxManifolds + k) * kTapeScalars;
                const uint32_t npts = sc.mCount[m];
                PointIn<S> ins[4];
                PointIn<S> s{ld3(tp, 0), ld3(tp, 1), ld3(tp, 2), ld3(tp, 3), z, z, z};
                for (uint32_t p = 0; p < npts; ++p) {
                    s.ln = tp[12 + 3 * p];
                    s.l1 = tp[12 + 3 * p + 1];
                    s.l2 = tp[12 + 3 * p + 2];
                    ins[p] = s;
                    pointForward(n3, mu, sc.pp + ((size_t)k * 4 + p) * kPreparedScalars, pm[18], pm[19], sA, sB, s);
                }
                PointIn<S> ab{sA ? V3<S>{z, z, z} : ld3(adj.av, a), sA ? V3<S>{z, z, z} : ld3(adj.aw, a),
                              sB ? V3<S>{z, z, z} : ld3(adj.av, b), sB ? V3<S>{z, z, z} : ld3(adj.aw, b), z, z, z};
                V3<S> an = ld3(adj.an, k);
                S amu = adj.amuM[k];
                S *apm = adj.apm + (size_t)k * kPmScalars;
                S aimA = apm[18], aimB = apm[19];
                for (int p = (int)npts - 1; p >= 0; --p) {
                    const size_t kp = (size_t)k * 4 + p;
                    ab.ln = adj.alam[3 * kp];
                    ab.l1 = adj.alam[3 * kp + 1];
                    ab.l2 = adj.alam[3 * kp + 2];
                    pointReverse(n3, mu, sc.pp + kp * kPreparedScalars, pm[18], pm[19], sA, sB, ins[p], ab,
                                 adj.app + kp * kPreparedScalars, an, amu, aimA, aimB);
                    adj.alam[3 * kp] = ab.ln;
                    adj.alam[3 * kp + 1] = ab.l1;
                    adj.alam[3 * kp + 2] = ab.l2;
                }
                apm[18] = aimA;
                apm[19] = aimB;
                st3(adj.an, k, an);
                adj.amuM[k] = amu;
                if (!sA) {
                    st3(adj.av, a, ab.vA);
                    st3(adj.aw, a, ab.wA);
                }
                if (!sB) {
                    st3(adj.av, b, ab.vB);
                    st3(adj.aw, b, ab.wB);
                }
            }
            T::sync();
        }
    // 3. warm start in reverse (additive: body adjoints pass through)
    for (uint32_t k = tid; k < M; k += nt) {
        const uint32_t m = sc.order[k];
        const uint32_t a = sc.mA[m], b = sc.mB[m];
        const bool sA = W.isStatic[a] != 0, sB = W.isStatic[b] != 0;
        const S *pm = sc.pm + (size_t)k * kPmScalars;
        S *apm = adj.apm + (size_t)k * kPmScalars;
        const M3<S> IA = ldm(pm), IB = ldm(pm + 9);
        const V3<S> n3 = ld3(sc.mNormal, m);
        const V3<S> avA = ld3(adj.av, a), awA = ld3(adj.aw, a), avB = ld3(adj.av, b), awB = ld3(adj.aw, b);
        V3<S> an = ld3(adj.an, k);
        for (uint32_t p = 0; p < sc.mCount[m]; ++p) {
            const size_t kp = (size_t)k * 4 + p;
            if (sc.match[kp] < 0) continue;
            const S *pp = sc.pp + kp * kPreparedScalars;
            S *ac = adj.app + kp * kPreparedScalars;
            const S ln = sc.lamInit[3 * kp], l1 = sc.lamInit[3 * kp + 1], l2 = sc.lamInit[3 * kp + 2];
            const V3<S> t1 = pv(pp, kPT1), t2 = pv(pp, kPT2), offA = pv(pp, kPOffA), offB = pv(pp, kPOffB);
            const V3<S> wi = n3 * ln + t1 * l1 + t2 * l2;
            const V3<S> nw = -wi;
            V3<S> awi{z, z, z};
            if (!sB) {
                awi += avB * pm[19];
                apm[19] = apm[19] + dot(avB, wi);
                const V3<S> y = cross(offB, wi);
                const V3<S> ay = mul(transpose(IB), awB);
                const S *yy = &y.x;
                const S *aww = &awB.x;
                for (int r = 0; r < 3; ++r)
                    for (int cc = 0; cc < 3; ++cc) apm[9 + 3 * r + cc] = apm[9 + 3 * r + cc] + aww[r] * yy[cc];
                V3<S> aoff{z, z, z};
                crossAdj(offB, wi, ay, aoff, awi);
                ac[3 * kPOffB] = ac[3 * kPOffB] + aoff.x;
                ac[3 * kPOffB + 1] = ac[3 * kPOffB + 1] + aoff.y;
                ac[3 * kPOffB + 2] = ac[3 * kPOffB + 2] + aoff.z;
            }
            if (!sA) {
                V3<S> anw = avA * pm[18];
                apm[18] = apm[18] + dot(avA, nw);
                const V3<S> y = cross(offA, nw);
                const V3<S> ay = mul(transpose(IA), awA);
                const S *yy = &y.x;
                const S *aww = &awA.x;
                for (int r = 0; r < 3; ++r)
                    for (int cc = 0; cc < 3; ++cc) apm[3 * r + cc] = apm[3 * r + cc] + aww[r] * yy[cc];
                V3<S> aoff{z, z, z};
                crossAdj(offA, nw, ay, aoff, anw);
                ac[3 * kPOffA] = ac[3 * kPOffA] + aoff.x;
                ac[3 * kPOffA + 1] = ac[3 * kPOffA + 1] + aoff.y;
                ac[3 * kPOffA + 2] = ac[3 * kPOffA + 2] + aoff.z;
                awi += -anw;
            }
            adj.alam[3 * kp] = adj.alam[3 * kp] + dot(awi, n3);
            adj.alam[3 * kp + 1] = adj.alam[3 * kp + 1] + dot(awi, t1);
            adj.alam[3 * kp + 2] = adj.alam[3 * kp + 2] + dot(awi, t2);
            an += awi * ln;
            ac[3 * kPT1] = ac[3 * kPT1] + awi.x * l1;
            ac[3 * kPT1 + 1] = ac[3 * kPT1 + 1] + awi.y * l1;
            ac[3 * kPT1 + 2] = ac[3 * kPT1 + 2] + awi.z * l1;
            ac[3 * kPT2] = ac[3 * kPT2] + awi.x * l2;
            ac[3 * kPT2 + 1] = ac[3 * kPT2 + 1] + awi.y * l2;
            ac[3 * kPT2 + 2] = ac[3 * kPT2 + 2] + awi.z * l2;
        }
        st3(adj.an, k, an);
        // 4. warm-start matching: lambda_init from the previous step's impulses
        const S mu = sc.mMu[m];
        S amu = adj.amuM[k];
        for (uint32_t p = 0; p < sc.mCount[m]; ++p) {
            const size_t kp = (size_t)k * 4 + p;
            const int32_t e = sc.match[kp];
            if (e < 0) continue;
            const S cn = cin.lam[3 * e], c1 = cin.lam[3 * e + 1], c2 = cin.lam[3 * e + 2];
            const S ni = smax(cn, z);
            const S mu0 = smax(mu, z);
            const S limit = mu0 * ni;
            const S tlsq = c1 * c1 + c2 * c2;
            S ani = adj.alam[3 * kp];
            const S af1 = adj.alam[3 * kp + 1], af2 = adj.alam[3 * kp + 2];
            S ac1 = af1, ac2 = af2;
            if (tlsq > limit * limit) {
                const S L = ssqrt(tlsq);
                const S u1 = c1 / L, u2 = c2 / L;
                const S ua = u1 * af1 + u2 * af2;
                ac1 = (limit / L) * (af1 - u1 * ua);
                ac2 = (limit / L) * (af2 - u2 * ua);
                ani = ani + ua * mu0;
                if (!(mu < z)) amu = amu + ua * ni;
            }
            const S acn = (cn < z) ? z : ani;
            T::add(&adj.acache[3 * e], acn);
            T::add(&adj.acache[3 * e + 1], ac1);
            T::add(&adj.acache[3 * e + 2], ac2);
        }
        adj.amuM[k] = amu;
    }
    T::sync();
    // 5. contact geometry + preparation (dual numbers): one (manifold, chunk of
    // four directions) per thread; 6. materials with the last chunk
    constexpr int kChunks = (kDualInputs + kDualChunk - 1) / kDualChunk;
    for (uint32_t item = tid; item < M * kChunks; item += nt) {
        const uint32_t k = item / kChunks;
        const int chunk = (int)(item % kChunks), base = chunk * kDualChunk;
        const uint32_t m = sc.order[k];
        const uint32_t a = sc.mA[m], b = sc.mB[m];
        const bool sA = W.isStatic[a] != 0, sB = W.isStatic[b] != 0;
        S gr[kDualChunk];
        if (!manifoldDualChunk(W, in, v1, sc, adj, k, base, gr)) {
            T::orErr(&sc.counts[3], kAdErrReplay);
            continue;
        }
        for (int j = 0; j < kDualChunk; ++j) {
            const int d = base + j;
            if (d >= kDualInputs) break;
            const S gv = gr[j];
            if (d < 3) {
                if (!sA) T::add(&adj.ax[3 * a + d], gv);
            } else if (d < 7) {
                if (!sA) T::add(&adj.aq[4 * a + (d - 3)], gv);
            } else if (d < 10) {
                if (!sB) T::add(&adj.ax[3 * b + (d - 7)], gv);
            } else if (d < 14) {
                if (!sB) T::add(&adj.aq[4 * b + (d - 10)], gv);
            } else if (d < 17) {
                if (!sA) T::add(&adj.av[3 * a + (d - 14)], gv);
            } else if (d < 20) {
                if (!sA) T::add(&adj.aw[3 * a + (d - 17)], gv);
            } else if (d < 23) {
                if (!sB) T::add(&adj.av[3 * b + (d - 20)], gv);
            } else if (d < 26) {
                if (!sB) T::add(&adj.aw[3 * b + (d - 23)], gv);
            } else if (d == 26) {
                if (!sA) T::add(&adj.amass[a], gv);
            } else if (d == 27) {
                if (!sB) T::add(&adj.amass[b], gv);
            } else {
                // restitution = max(ra, rb)
                const S arest = adj.arestM[k] + gv;
                if (W.rest[a] < W.rest[b]) {
                    if (!sB) T::add(&adj.arest[b], arest);
                } else if (!sA) {
                    T::add(&adj.arest[a], arest);
                }
            }
        }
        if (chunk == 0) {
            // friction = sqrt(max(fa, 0) * max(fb, 0))
            const S fm = sc.mMu[m];
            if (fm > z) {
                const S fa = smax(W.mu[a], z), fb = smax(W.mu[b], z);
                const S amu = adj.amuM[k] * (S(0.5f) / fm);
                if (!sA && !(W.mu[a] < z)) T::add(&adj.amu[a], amu * fb);
                if (!sB && !(W.mu[b] < z)) T::add(&adj.amu[b], amu * fa);
            }
        }
    }
    T::sync();
}

} // namespace ad
} // namespace pe
