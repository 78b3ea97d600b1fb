// Device narrowphase: one call produces one contact manifold for one collider
// pair.  Operation order follows src/collision/narrowphase.cpp (sphere-sphere
// :132-160, sphere-box :162-248, box-box :250-324, dispatch/swap :326-374) and
// src/collision/sat.cpp:38-102, so results are bit-identical to the reference
// under --fmad=false.  Feature ids (which the reference lacks) are
// (kind << 24) | (source << 16) | (face axis << 8) | (face sign << 4) | vertex.
// Convex hulls go through GJK (src/collision/gjk.cpp:11-158) and EPA
// (src/collision/epa.cpp:29-130) over support maps, with bounded polytope storage.
#pragma once
#include "pe_engine.h"
#include "pe_math.cuh"

namespace pe {

struct LocalManifold {
    V3 normal;
    uint32_t count;
    V3 anchorA[4];
    V3 anchorB[4];
    float depth[4];
    uint32_t feature[4];
};

__device__ __forceinline__ V3 boxSupport(const V3 &he, const Tf &tf, const V3 &dir) {
    V3 ld = rotate(conj(tf.q), dir);
    V3 lp{ld.x >= 0.0f ? he.x : -he.x, ld.y >= 0.0f ? he.y : -he.y, ld.z >= 0.0f ? he.z : -he.z};
    return toWorld(lp, tf);
}

__device__ __forceinline__ float boxProjectedRadius(const V3 &he, const M3 &r, const V3 &axis) {
    V3 a0{r.m00, r.m10, r.m20}, a1{r.m01, r.m11, r.m21}, a2{r.m02, r.m12, r.m22};
    return fabsf(dot(a0, axis)) * he.x + fabsf(dot(a1, axis)) * he.y + fabsf(dot(a2, axis)) * he.z;
}

// intersectSphereSphere (narrowphase.cpp:132-160)
__device__ __forceinline__ bool sphereSphere(float rA, const Tf &tA, float rB, const Tf &tB, LocalManifold &m) {
    V3 delta = tB.p - tA.p;
    float distance = length(delta);
    float radii = rA + rB;
    if (distance >= radii) return false;
    m.normal = distance > 1e-6f ? delta / distance : V3{1.0f, 0.0f, 0.0f};
    m.count = 1;
    m.depth[0] = radii - distance;
    V3 pA = tA.p + m.normal * rA;
    V3 pB = tB.p - m.normal * rB;
    V3 wc = (pA + pB) * 0.5f;
    m.anchorA[0] = toLocal(wc, tA);
    m.anchorB[0] = toLocal(wc, tB);
    m.feature[0] = kFeatSphereSphere << 24;
    return true;
}

// intersectSphereBox (narrowphase.cpp:162-248); region: 0..5 nearest face when
// the centre is inside, 6 outside.
__device__ __forceinline__ bool sphereBox(float r, const Tf &tS, const V3 &he, const Tf &tB, LocalManifold &m) {
    V3 c = rotate(conj(tB.q), tS.p - tB.p);
    V3 cl{clampv(c.x, -he.x, he.x), clampv(c.y, -he.y, he.y), clampv(c.z, -he.z, he.z)};
    V3 dl = cl - c;
    float distance = length(dl);
    V3 nl;
    float pen;
    uint32_t region;
    if (distance > 1e-6f) {
        if (distance >= r) return false;
        nl = dl / distance;
        pen = r - distance;
        region = 6;
    } else {
        float dpx = he.x - c.x, dnx = he.x + c.x, dpy = he.y - c.y, dny = he.y + c.y, dpz = he.z - c.z,
              dnz = he.z + c.z;
        float nearest = dpx;
        nl = {-1.0f, 0.0f, 0.0f};
        region = 0;
        if (dnx < nearest) { nearest = dnx; nl = {1.0f, 0.0f, 0.0f}; region = 1; }
        if (dpy < nearest) { nearest = dpy; nl = {0.0f, -1.0f, 0.0f}; region = 2; }
        if (dny < nearest) { nearest = dny; nl = {0.0f, 1.0f, 0.0f}; region = 3; }
        if (dpz < nearest) { nearest = dpz; nl = {0.0f, 0.0f, -1.0f}; region = 4; }
        if (dnz < nearest) { nearest = dnz; nl = {0.0f, 0.0f, 1.0f}; region = 5; }
        pen = r + nearest;
    }
    m.normal = rotate(tB.q, nl);
    m.count = 1;
    m.depth[0] = pen;
    V3 bp = toWorld(cl, tB);
    V3 sp = tS.p + m.normal * r;
    V3 wc = (sp + bp) * 0.5f;
    m.anchorA[0] = toLocal(wc, tS);
    m.anchorB[0] = toLocal(wc, tB);
    m.feature[0] = (kFeatSphereBox << 24) | region;
    return true;
}

// overlapOnAxis (sat.cpp:45-62); axes of a box are the columns of its matrix.
__device__ __forceinline__ bool satAxis(const M3 &rA, const V3 &heA, const M3 &rB, const V3 &heB, const V3 &cd,
                                        const V3 &axis, V3 &bestAxis, float &bestDepth) {
    float lsq = dot(axis, axis);
    if (lsq < 1e-8f) return true; // degenerate axis: depth = FLT_MAX never wins
    V3 na = axis * (1.0f / sqrtf(lsq));
    float distance = fabsf(dot(cd, na));
    float d = (boxProjectedRadius(heA, rA, na) + boxProjectedRadius(heB, rB, na)) - distance;
    if (d < 0.0f) return false;
    if (d < bestDepth) {
        bestDepth = d;
        bestAxis = na;
    }
    return true;
}

// Column j of a rotation matrix (a box's local axis j in world space).
__device__ __forceinline__ V3 matColumn(const M3 &r, int j) {
    return j == 0 ? V3{r.m00, r.m10, r.m20} : j == 1 ? V3{r.m01, r.m11, r.m21} : V3{r.m02, r.m12, r.m22};
}

// testOBBOBB (sat.cpp:66-102): face axes of A, of B, then A_i x B_j, in that
// order.  One rolled loop over the 15 axes: the kernel runs this once per pair,
// so a single copy of the axis test (fetched once) beats 15 unrolled copies.
__device__ __forceinline__ bool satBoxBox(const V3 &heA, const Tf &tA, const M3 &rA, const V3 &heB, const Tf &tB,
                                          const M3 &rB, V3 &axis, float &depth) {
    depth = 3.402823466e+38f;
    V3 cd = tB.p - tA.p;
#pragma unroll 1
    for (int t = 0; t < 15; ++t) {
        V3 ax;
        if (t < 3) ax = matColumn(rA, t);
        else if (t < 6) ax = matColumn(rB, t - 3);
        else ax = cross(matColumn(rA, (t - 6) / 3), matColumn(rB, (t - 6) % 3));
        if (!satAxis(rA, heA, rB, heB, cd, ax, axis, depth)) return false;
    }
    return true;
}

// addFaceCandidates (narrowphase.cpp:281-304) for one source box face.
// (not inlined: its two calls per box pair share one copy of the code)
static __device__ __noinline__ void boxFaceCandidates(const V3 &srcHe, const Tf &srcTf, const V3 &othHe, const Tf &othTf,
                                                  const V3 &dir, uint32_t source, V3 *contacts, float *depths,
                                                  uint32_t *feats, uint32_t &count) {
    float otherSurface = dot(boxSupport(othHe, othTf, -dir), dir);
    // supportFaceVertices (narrowphase.cpp:60-98)
    V3 ld = rotate(conj(srcTf.q), dir);
    int faceAxis = 0;
    float largest = fabsf(ld.x);
    if (fabsf(ld.y) > largest) { faceAxis = 1; largest = fabsf(ld.y); }
    if (fabsf(ld.z) > largest) faceAxis = 2;
    float comp = faceAxis == 0 ? ld.x : faceAxis == 1 ? ld.y : ld.z;
    float faceSign = comp >= 0.0f ? 1.0f : -1.0f;
    uint32_t signBit = comp >= 0.0f ? 0u : 1u;
    float ext[3] = {srcHe.x, srcHe.y, srcHe.z};
    int fa = (faceAxis + 1) % 3, sa = (faceAxis + 2) % 3;
    Q cq = conj(othTf.q);
    for (uint32_t vi = 0; vi < 4; ++vi) {
        float c[3] = {0.0f, 0.0f, 0.0f};
        c[faceAxis] = faceSign * ext[faceAxis];
        c[fa] = (vi & 1) ? ext[fa] : -ext[fa];
        c[sa] = (vi & 2) ? ext[sa] : -ext[sa];
        V3 v = toWorld(V3{c[0], c[1], c[2]}, srcTf);
        // pointInsideBox (narrowphase.cpp:100-107)
        V3 l = rotate(cq, v - othTf.p);
        const float tol = 1e-4f;
        if (!(fabsf(l.x) <= othHe.x + tol && fabsf(l.y) <= othHe.y + tol && fabsf(l.z) <= othHe.z + tol)) continue;
        float depth = smax(dot(v, dir) - otherSurface, 0.0f);
        V3 cand = v - dir * (depth * 0.5f);
        if (count >= 4) continue;
        // duplicatePoint (narrowphase.cpp:109-120)
        bool dup = false;
        for (uint32_t k = 0; k < count; ++k) {
            V3 dd = contacts[k] - cand;
            if (dot(dd, dd) <= 1e-6f) dup = true;
        }
        if (dup) continue;
        depths[count] = depth;
        feats[count] = (kFeatBoxFace << 24) | (source << 16) | ((uint32_t)faceAxis << 8) | (signBit << 4) | vi;
        contacts[count++] = cand;
    }
}

// intersectBoxBox (narrowphase.cpp:250-324)
__device__ __forceinline__ bool boxBox(const V3 &heA, const Tf &tA, const V3 &heB, const Tf &tB, LocalManifold &m) {
    M3 rA = toMat3(tA.q), rB = toMat3(tB.q);
    V3 normal;
    float penetration;
    if (!satBoxBox(heA, tA, rA, heB, tB, rB, normal, penetration)) return false;
    V3 cd = tB.p - tA.p;
    if (dot(cd, normal) < 0.0f) normal = -normal;
    m.normal = normal;
    V3 contacts[4];
    float depths[4];
    uint32_t feats[4];
    uint32_t count = 0;
    boxFaceCandidates(heA, tA, heB, tB, normal, 0, contacts, depths, feats, count);
    boxFaceCandidates(heB, tB, heA, tA, -normal, 1, contacts, depths, feats, count);
    if (count == 0) {
        // Fallback contact (narrowphase.cpp:270-276, 308-312).
        V3 tref = fabsf(normal.x) < 0.9f ? V3{1.0f, 0.0f, 0.0f} : V3{0.0f, 1.0f, 0.0f};
        V3 t1 = normalize(cross(normal, tref));
        V3 t2 = cross(normal, t1);
        float nc = (dot(tA.p, normal) + boxProjectedRadius(heA, rA, normal) + dot(tB.p, normal) -
                    boxProjectedRadius(heB, rB, normal)) *
                   0.5f;
        // overlapMidpoint (narrowphase.cpp:48-58)
        auto mid = [&](const V3 &ax) {
            float cA = dot(tA.p, ax), cB = dot(tB.p, ax);
            float ra = boxProjectedRadius(heA, rA, ax), rb = boxProjectedRadius(heB, rB, ax);
            float lower = smax(cA - ra, cB - rb);
            float upper = smin(cA + ra, cB + rb);
            return (lower + upper) * 0.5f;
        };
        contacts[0] = normal * nc + t1 * mid(t1) + t2 * mid(t2);
        depths[0] = penetration;
        feats[0] = kFeatBoxFallback << 24;
        count = 1;
    }
    m.count = count;
    for (uint32_t i = 0; i < count; ++i) {
        m.depth[i] = depths[i];
        m.anchorA[i] = toLocal(contacts[i], tA);
        m.anchorB[i] = toLocal(contacts[i], tB);
        m.feature[i] = feats[i];
    }
    return true;
}

// ---------------------------------------------------------------------------
// GJK / EPA over support maps (box: boxSupportPoint; sphere: centre +
// normalize(d) * r; hull: first vertex of maximal d . v in body space).
// ---------------------------------------------------------------------------
constexpr int kEpaMaxVertices = 4 + 64;
constexpr int kEpaMaxFaces = 256;
constexpr int kEpaMaxHorizon = 128;

struct SupportShape {
    uint32_t shape;
    float radius;
    V3 he;
    const float4 *verts;
    uint32_t nverts;
    Tf tf;
};

__device__ __forceinline__ V3 support(const SupportShape &s, const V3 &dir, uint32_t &index) {
    if (s.shape == kShapeBox) return boxSupport(s.he, s.tf, dir);
    if (s.shape == kShapeSphere) return s.tf.p + normalize(dir) * s.radius;
    V3 ld = rotate(conj(s.tf.q), dir);
    uint32_t best = 0;
    float4 v0 = s.verts[0];
    float bd = dot(V3{v0.x, v0.y, v0.z}, ld);
    for (uint32_t i = 1; i < s.nverts; ++i) {
        float4 v = s.verts[i];
        float d = dot(V3{v.x, v.y, v.z}, ld);
        if (d > bd) { bd = d; best = i; }
    }
    index = best;
    float4 vb = s.verts[best];
    return toWorld(V3{vb.x, vb.y, vb.z}, s.tf);
}

struct Simplex {
    V3 p[4];
    uint32_t size;
};

__device__ __forceinline__ V3 tripleCross(const V3 &a, const V3 &b, const V3 &c) { return cross(cross(a, b), c); }

// setLineDirection (gjk.cpp:21-41)
__device__ inline void gjkLine(Simplex &s, V3 &dir) {
    V3 A = s.p[0], B = s.p[1];
    V3 toO = -A;
    V3 e = B - A;
    if (dot(e, toO) > 0.0f) {
        dir = tripleCross(e, toO, e);
        if (dot(dir, dir) < 1e-12f) dir = cross(e, V3{1.0f, 0.0f, 0.0f});
        if (dot(dir, dir) < 1e-12f) dir = cross(e, V3{0.0f, 1.0f, 0.0f});
    } else {
        s.size = 1;
        dir = toO;
    }
}
// setTriangleDirection (gjk.cpp:43-74)
__device__ inline void gjkTriangle(Simplex &s, V3 &dir) {
    V3 A = s.p[0], B = s.p[1], C = s.p[2];
    V3 toO = -A;
    V3 ab = B - A, ac = C - A;
    V3 n = cross(ab, ac);
    if (dot(cross(n, ac), toO) > 0.0f) {
        if (dot(ac, toO) > 0.0f) {
            s.p[1] = C;
            s.size = 2;
            dir = tripleCross(ac, toO, ac);
            return;
        }
        gjkLine(s, dir);
        return;
    }
    if (dot(cross(ab, n), toO) > 0.0f) {
        gjkLine(s, dir);
        return;
    }
    if (dot(n, toO) > 0.0f) {
        dir = n;
    } else {
        V3 t = s.p[1];
        s.p[1] = s.p[2];
        s.p[2] = t;
        dir = -n;
    }
}
// containsOrigin (gjk.cpp:76-124), including its third-face assignment through
// aliased references (the simplex becomes {A, D, D}).
__device__ inline bool gjkContains(Simplex &s, V3 &dir) {
    if (s.size == 1) {
        dir = -s.p[0];
        return false;
    }
    if (s.size == 2) {
        gjkLine(s, dir);
        return false;
    }
    if (s.size == 3) {
        gjkTriangle(s, dir);
        return false;
    }
    V3 A = s.p[0];
    V3 toO = -A;
    auto outside = [&](const V3 &fb, const V3 &fc, const V3 &op) {
        V3 n = cross(fb - A, fc - A);
        if (dot(n, op - A) > 0.0f) n = -n;
        return dot(n, toO) > 0.0f;
    };
    if (outside(s.p[1], s.p[2], s.p[3])) {
        s.size = 3;
        gjkTriangle(s, dir);
        return false;
    }
    if (outside(s.p[2], s.p[3], s.p[1])) {
        s.p[1] = s.p[2];
        s.p[2] = s.p[3];
        s.size = 3;
        gjkTriangle(s, dir);
        return false;
    }
    if (outside(s.p[3], s.p[1], s.p[2])) {
        s.p[1] = s.p[3];
        s.p[2] = s.p[1];
        s.size = 3;
        gjkTriangle(s, dir);
        return false;
    }
    return true;
}

__device__ inline bool gjk(const SupportShape &A, const SupportShape &B, Simplex &s) {
    s.size = 0;
    V3 dir{1.0f, 0.0f, 0.0f};
    uint32_t ia, ib;
    for (uint32_t it = 0; it < 32; ++it) {
        if (dot(dir, dir) < 1e-12f) break;
        V3 p = support(A, dir, ia) - support(B, -dir, ib);
        if (dot(p, dir) <= 0.0f) break;
        for (uint32_t i = s.size < 3u ? s.size : 3u; i > 0; --i) s.p[i] = s.p[i - 1];
        s.p[0] = p;
        s.size = s.size + 1 < 4u ? s.size + 1 : 4u;
        if (gjkContains(s, dir)) return true;
    }
    return false;
}

struct EpaFace {
    uint16_t a, b, c;
    V3 n;
    float d;
};

__device__ __forceinline__ EpaFace epaFace(const V3 *v, uint32_t a, uint32_t b, uint32_t c) {
    V3 n = cross(v[b] - v[a], v[c] - v[a]);
    float len = length(n);
    if (len > 1e-8f) n = n * (1.0f / len);
    float d = dot(n, v[a]);
    if (d < 0.0f) {
        uint32_t t = b;
        b = c;
        c = t;
        n = -n;
        d = -d;
    }
    return {(uint16_t)a, (uint16_t)b, (uint16_t)c, n, d};
}

// computeEpa (epa.cpp:64-130); 1 on success, 0 on failure (degenerate,
// iteration cap, or bounded storage exhausted).  Storage is per thread.
__device__ inline int epa(const SupportShape &A, const SupportShape &B, const Simplex &s, V3 &normal, float &depth) {
    normal = V3{0.0f, 0.0f, 0.0f};
    depth = 0.0f;
    if (s.size < 4) return 0;
    V3 v[kEpaMaxVertices];
    EpaFace faces[kEpaMaxFaces];
    uint16_t he[kEpaMaxHorizon][2];
    uint32_t nv = 0, nf = 0;
    for (uint32_t i = 0; i < s.size; ++i) v[nv++] = s.p[i];
    faces[nf++] = epaFace(v, 0, 1, 2);
    faces[nf++] = epaFace(v, 0, 3, 1);
    faces[nf++] = epaFace(v, 0, 2, 3);
    faces[nf++] = epaFace(v, 1, 3, 2);
    const float tol = 1e-4f;
    uint32_t ia, ib;
    for (uint32_t it = 0; it < 64; ++it) {
        if (nf == 0) return 0;
        uint32_t ci = 0;
        for (uint32_t f = 1; f < nf; ++f)
            if (faces[f].d < faces[ci].d) ci = f;
        EpaFace cf = faces[ci];
        V3 sup = support(A, cf.n, ia) - support(B, -cf.n, ib);
        float sd = dot(sup, cf.n);
        if (sd - cf.d <= tol) {
            normal = cf.n;
            depth = smax(cf.d, 0.0f);
            return 1;
        }
        if (nv >= (uint32_t)kEpaMaxVertices) return 0;
        uint32_t si = nv;
        v[nv++] = sup;
        uint32_t nh = 0;
        bool overflow = false;
        uint32_t kept = 0;
        for (uint32_t f = 0; f < nf; ++f) {
            const EpaFace face = faces[f];
            float vis = dot(face.n, sup - v[face.a]);
            if (vis > tol) {
                uint32_t e[3][2] = {{face.a, face.b}, {face.b, face.c}, {face.c, face.a}};
                for (int k = 0; k < 3; ++k) {
                    uint32_t a = e[k][0], b = e[k][1];
                    bool removed = false;
                    for (uint32_t q = 0; q < nh; ++q)
                        if (he[q][0] == b && he[q][1] == a) {
                            for (uint32_t r = q + 1; r < nh; ++r) {
                                he[r - 1][0] = he[r][0];
                                he[r - 1][1] = he[r][1];
                            }
                            --nh;
                            removed = true;
                            break;
                        }
                    if (!removed) {
                        if (nh >= (uint32_t)kEpaMaxHorizon) {
                            overflow = true;
                        } else {
                            he[nh][0] = (uint16_t)a;
                            he[nh][1] = (uint16_t)b;
                            ++nh;
                        }
                    }
                }
            } else {
                faces[kept++] = face;
            }
        }
        if (overflow || nh == 0) return 0;
        nf = kept;
        if (nf + nh > (uint32_t)kEpaMaxFaces) return 0;
        for (uint32_t k = 0; k < nh; ++k) faces[nf++] = epaFace(v, he[k][0], he[k][1], si);
    }
    return 0;
}

// Hull contact (project-defined): normal and depth from EPA (A toward B), one
// point midway between A's support along n and B's support along -n.
__device__ inline bool hullContact(const SupportShape &A, const SupportShape &B, LocalManifold &m, bool &epaFailed) {
    epaFailed = false;
    Simplex s;
    if (!gjk(A, B, s)) return false;
    V3 n;
    float depth;
    if (!epa(A, B, s, n, depth)) {
        epaFailed = true;
        return false;
    }
    uint32_t ia = 0xFFu, ib = 0xFFu;
    V3 pa = support(A, n, ia);
    V3 pb = support(B, -n, ib);
    if (A.shape != kShapeHull) ia = 0xFFu;
    if (B.shape != kShapeHull) ib = 0xFFu;
    V3 wc = (pa + pb) * 0.5f;
    m.normal = n;
    m.count = 1;
    m.depth[0] = depth;
    m.anchorA[0] = toLocal(wc, A.tf);
    m.anchorB[0] = toLocal(wc, B.tf);
    m.feature[0] = (kFeatHull << 24) | ((ia & 0xFFu) << 8) | (ib & 0xFFu);
    return true;
}


__device__ inline SupportShape supportShape(const WorldView &w, uint32_t c, const Tf &t) {
    SupportShape s;
    s.shape = colliderShape(w.cflags[c]);
    float4 sh = w.cshape[c];
    s.radius = sh.x;
    s.he = V3{sh.x, sh.y, sh.z};
    s.tf = t;
    s.verts = nullptr;
    s.nverts = 0;
    if (s.shape == kShapeHull) {
        uint32_t h = __float_as_uint(sh.w);
        uint32_t b = w.hullOffset[h];
        s.verts = w.hullVerts + b;
        s.nverts = w.hullOffset[h + 1] - b;
    }
    return s;
}

// The world's generateContact lambda (src/world/physics_world.cpp:645-691) for
// collider slots ca, cb of bodies ba, bb: world transforms, shape dispatch with
// the box-sphere swap (narrowphase.cpp:353-365), anchors to body space,
// restitution = max, friction = sqrt(max(fa,0) * max(fb,0)).  category: 0
// sphere-sphere, 1 sphere-box, 2 box-box, 3 hull.
__device__ inline bool narrowphasePair(const WorldView &w, uint32_t ca, uint32_t cb, uint32_t ba, uint32_t bb,
                                       LocalManifold &lm, float &restitution, float &friction, uint32_t &category,
                                       bool &epaFailed) {
    epaFailed = false;
    lm.count = 0;
    const uint32_t sa = colliderShape(w.cflags[ca]), sb = colliderShape(w.cflags[cb]);
    V3 lpa = w.clpos ? f4xyz(w.clpos[ca]) : V3{0.0f, 0.0f, 0.0f};
    Q lqa = w.clrot ? f4q(w.clrot[ca]) : qidentity();
    V3 lpb = w.clpos ? f4xyz(w.clpos[cb]) : V3{0.0f, 0.0f, 0.0f};
    Q lqb = w.clrot ? f4q(w.clrot[cb]) : qidentity();
    V3 pa = f4xyz(w.cur.pos[ba]), pb = f4xyz(w.cur.pos[bb]);
    Q qa = f4q(w.cur.rot[ba]), qb = f4q(w.cur.rot[bb]);
    Tf tA{pa + rotate(qa, lpa), qmul(qa, lqa)};
    Tf tB{pb + rotate(qb, lpb), qmul(qb, lqb)};
    const float4 sha = w.cshape[ca], shb = w.cshape[cb];
    bool hit;
    if (sa == kShapeHull || sb == kShapeHull) {
        category = 3;
        hit = hullContact(supportShape(w, ca, tA), supportShape(w, cb, tB), lm, epaFailed);
    } else {
        category = sa + sb;
        if (sa == kShapeSphere && sb == kShapeSphere) {
            hit = sphereSphere(sha.x, tA, shb.x, tB, lm);
        } else if (sa == kShapeSphere) {
            hit = sphereBox(sha.x, tA, V3{shb.x, shb.y, shb.z}, tB, lm);
        } else if (sb == kShapeSphere) {
            hit = sphereBox(shb.x, tB, V3{sha.x, sha.y, sha.z}, tA, lm);
            if (hit) {
                lm.normal = -lm.normal;
                for (uint32_t k = 0; k < lm.count; ++k) {
                    V3 t = lm.anchorA[k];
                    lm.anchorA[k] = lm.anchorB[k];
                    lm.anchorB[k] = t;
                }
            }
        } else {
            hit = boxBox(V3{sha.x, sha.y, sha.z}, tA, V3{shb.x, shb.y, shb.z}, tB, lm);
        }
    }
    if (hit) {
        for (uint32_t k = 0; k < lm.count; ++k) {
            lm.anchorA[k] = lpa + rotate(lqa, lm.anchorA[k]);
            lm.anchorB[k] = lpb + rotate(lqb, lm.anchorB[k]);
        }
        const float4 ma = w.mat[ba], mb = w.mat[bb];
        restitution = smax(ma.y, mb.y);
        friction = sqrtf(smax(ma.z, 0.0f) * smax(mb.z, 0.0f));
    }
    return hit;
}

// narrowphasePair with both colliders read from their packed records
// (WorldView::npRec, written by the integrate kernel with the same world
// transforms, shapes and materials): one 64-byte line per collider instead of
// a gather from a dozen arrays.  ra / rb: the four float4 of each record.
__device__ inline bool narrowphasePairRec(const WorldView &w, uint32_t ca, uint32_t cb, const float4 *ra,
                                          const float4 *rb, LocalManifold &lm, float &restitution, float &friction,
                                          uint32_t &category, bool &epaFailed) {
    epaFailed = false;
    lm.count = 0;
    const uint32_t sa = colliderShape(__float_as_uint(ra[2].w)), sb = colliderShape(__float_as_uint(rb[2].w));
    const Tf tA{V3{ra[0].x, ra[0].y, ra[0].z}, Q{ra[1].x, ra[1].y, ra[1].z, ra[1].w}};
    const Tf tB{V3{rb[0].x, rb[0].y, rb[0].z}, Q{rb[1].x, rb[1].y, rb[1].z, rb[1].w}};
    const float4 sha = make_float4(ra[0].w, ra[2].x, ra[2].y, ra[2].z);
    const float4 shb = make_float4(rb[0].w, rb[2].x, rb[2].y, rb[2].z);
    bool hit;
    if (sa == kShapeHull || sb == kShapeHull) {
        category = 3;
        auto support = [&](uint32_t shape, const float4 &sh, const Tf &t) {
            SupportShape s;
            s.shape = shape;
            s.radius = sh.x;
            s.he = V3{sh.x, sh.y, sh.z};
            s.tf = t;
            s.verts = nullptr;
            s.nverts = 0;
            if (shape == kShapeHull) {
                const uint32_t h = __float_as_uint(sh.w);
                const uint32_t b = w.hullOffset[h];
                s.verts = w.hullVerts + b;
                s.nverts = w.hullOffset[h + 1] - b;
            }
            return s;
        };
        hit = hullContact(support(sa, sha, tA), support(sb, shb, tB), lm, epaFailed);
    } else {
        category = sa + sb;
        if (sa == kShapeSphere && sb == kShapeSphere) {
            hit = sphereSphere(sha.x, tA, shb.x, tB, lm);
        } else if (sa == kShapeSphere) {
            hit = sphereBox(sha.x, tA, V3{shb.x, shb.y, shb.z}, tB, lm);
        } else if (sb == kShapeSphere) {
            hit = sphereBox(shb.x, tB, V3{sha.x, sha.y, sha.z}, tA, lm);
            if (hit) {
                lm.normal = -lm.normal;
                for (uint32_t k = 0; k < lm.count; ++k) {
                    V3 t = lm.anchorA[k];
                    lm.anchorA[k] = lm.anchorB[k];
                    lm.anchorB[k] = t;
                }
            }
        } else {
            hit = boxBox(V3{sha.x, sha.y, sha.z}, tA, V3{shb.x, shb.y, shb.z}, tB, lm);
        }
    }
    if (hit) {
        // anchors from collider space to body space (local transforms only
        // when some collider has one)
        const V3 lpa = w.clpos ? f4xyz(w.clpos[ca]) : V3{0.0f, 0.0f, 0.0f};
        const Q lqa = w.clrot ? f4q(w.clrot[ca]) : qidentity();
        const V3 lpb = w.clpos ? f4xyz(w.clpos[cb]) : V3{0.0f, 0.0f, 0.0f};
        const Q lqb = w.clrot ? f4q(w.clrot[cb]) : qidentity();
        for (uint32_t k = 0; k < lm.count; ++k) {
            lm.anchorA[k] = lpa + rotate(lqa, lm.anchorA[k]);
            lm.anchorB[k] = lpb + rotate(lqb, lm.anchorB[k]);
        }
        restitution = smax(ra[3].x, rb[3].x);
        friction = sqrtf(smax(ra[3].y, 0.0f) * smax(rb[3].y, 0.0f));
    }
    return hit;
}

// Writes one manifold record in pair order: body handles, collider-space
// anchors already moved to body space, zero impulses.
__device__ __forceinline__ void storeManifoldGen(const ManifoldView &out, uint32_t m, uint32_t ba, uint32_t genA,
                                                 uint32_t bb, uint32_t genB, const LocalManifold &lm,
                                                 float restitution, float friction) {
    out.bodyA[m] = ba;
    out.genA[m] = genA;
    out.bodyB[m] = bb;
    out.genB[m] = genB;
    out.normalFriction[m] = make4(lm.normal, friction);
    out.restitution[m] = restitution;
    out.pointCount[m] = lm.count;
    for (uint32_t k = 0; k < 4; ++k) {
        const bool live = k < lm.count;
        out.anchorA[4 * m + k] = live ? make4(lm.anchorA[k], lm.depth[k]) : make_float4(0, 0, 0, 0);
        out.anchorB[4 * m + k] = live ? make4(lm.anchorB[k], 0.0f) : make_float4(0, 0, 0, 0);
        out.impulse[4 * m + k] = make_float4(0, 0, 0, 0);
        out.feature[4 * m + k] = live ? lm.feature[k] : 0u;
    }
}

// storeManifold with the body handles taken from the colliders.
__device__ __forceinline__ void storeManifold(const ManifoldView &out, uint32_t m, const WorldView &w, uint32_t ca,
                                              uint32_t cb, uint32_t ba, uint32_t bb, const LocalManifold &lm,
                                              float restitution, float friction) {
    storeManifoldGen(out, m, ba, w.cbgen[ca], bb, w.cbgen[cb], lm, restitution, friction);
}

} // namespace pe
