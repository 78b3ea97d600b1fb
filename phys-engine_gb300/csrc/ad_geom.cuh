// Scalar-generic contact geometry and contact preparation for the
// differentiable rollout (sphere / box colliders, one per body, identity local
// transforms).  The operations mirror the engine's device narrowphase and
// prepare step, which follow src/collision/narrowphase.cpp (sphere-sphere
// :132-160, sphere-box :162-248, box-box :250-324, dispatch :326-374),
// src/collision/sat.cpp:38-102 and sequential_impulse_solver.cpp:101-214.
// Discrete choices (separating axis, kept vertices, clamps) are taken on the
// values, so a dual-number evaluation differentiates the contact the plain
// evaluation produced with those choices held.
#pragma once
#include "ad_math.cuh"

namespace pe {
namespace ad {

enum : uint32_t { kAdFeatSphereSphere = 1, kAdFeatSphereBox = 2, kAdFeatBoxFace = 3, kAdFeatBoxFallback = 4 };

template <class S> struct Contact {
    V3<S> normal;
    uint32_t count;
    V3<S> anchorA[4];
    V3<S> anchorB[4];
    S depth[4];
    uint32_t feature[4];
};

template <class S> AD_HD V3<S> cst(float x, float y, float z) { return {ADL(S, x), ADL(S, y), ADL(S, z)}; }

template <class S> AD_HD V3<S> boxSupport(const V3<S> &he, const Tf<S> &tf, const V3<S> &dir) {
    V3<S> ld = rotate(conj(tf.q), dir);
    V3<S> lp{val(ld.x) >= 0.0f ? he.x : -he.x, val(ld.y) >= 0.0f ? he.y : -he.y, val(ld.z) >= 0.0f ? he.z : -he.z};
    return toWorld(lp, tf);
}

template <class S> AD_HD S boxProjectedRadius(const V3<S> &he, const M3<S> &r, const V3<S> &axis) {
    V3<S> a0{r.m00, r.m10, r.m20}, a1{r.m01, r.m11, r.m21}, a2{r.m02, r.m12, r.m22};
    return sabs(dot(a0, axis)) * he.x + sabs(dot(a1, axis)) * he.y + sabs(dot(a2, axis)) * he.z;
}

// intersectSphereSphere (narrowphase.cpp:132-160)
template <class S>
AD_HDN bool sphereSphere(const S &rA, const Tf<S> &tA, const S &rB, const Tf<S> &tB, Contact<S> &m) {
    V3<S> delta = tB.p - tA.p;
    S distance = length(delta);
    S radii = rA + rB;
    if (val(distance) >= val(radii)) return false;
    m.normal = val(distance) > 1e-6f ? delta / distance : cst<S>(1.0f, 0.0f, 0.0f);
    m.count = 1;
    m.depth[0] = radii - distance;
    V3<S> pA = tA.p + m.normal * rA;
    V3<S> pB = tB.p - m.normal * rB;
    V3<S> wc = (pA + pB) * ADL(S, 0.5f);
    m.anchorA[0] = toLocal(wc, tA);
    m.anchorB[0] = toLocal(wc, tB);
    m.feature[0] = kAdFeatSphereSphere << 24;
    return true;
}

// intersectSphereBox (narrowphase.cpp:162-248)
template <class S>
AD_HDN bool sphereBox(const S &r, const Tf<S> &tS, const V3<S> &he, const Tf<S> &tB, Contact<S> &m) {
    V3<S> c = rotate(conj(tB.q), tS.p - tB.p);
    V3<S> cl{clampv(c.x, -he.x, he.x), clampv(c.y, -he.y, he.y), clampv(c.z, -he.z, he.z)};
    V3<S> dl = cl - c;
    S distance = length(dl);
    V3<S> nl;
    S pen;
    uint32_t region;
    if (val(distance) > 1e-6f) {
        if (val(distance) >= val(r)) return false;
        nl = dl / distance;
        pen = r - distance;
        region = 6;
    } else {
        S dpx = he.x - c.x, dnx = he.x + c.x, dpy = he.y - c.y, dny = he.y + c.y, dpz = he.z - c.z, dnz = he.z + c.z;
        S nearest = dpx;
        nl = cst<S>(-1.0f, 0.0f, 0.0f);
        region = 0;
        if (val(dnx) < val(nearest)) { nearest = dnx; nl = cst<S>(1.0f, 0.0f, 0.0f); region = 1; }
        if (val(dpy) < val(nearest)) { nearest = dpy; nl = cst<S>(0.0f, -1.0f, 0.0f); region = 2; }
        if (val(dny) < val(nearest)) { nearest = dny; nl = cst<S>(0.0f, 1.0f, 0.0f); region = 3; }
        if (val(dpz) < val(nearest)) { nearest = dpz; nl = cst<S>(0.0f, 0.0f, -1.0f); region = 4; }
        if (val(dnz) < val(nearest)) { nearest = dnz; nl = cst<S>(0.0f, 0.0f, 1.0f); region = 5; }
        pen = r + nearest;
    }
    m.normal = rotate(tB.q, nl);
    m.count = 1;
    m.depth[0] = pen;
    V3<S> bp = toWorld(cl, tB);
    V3<S> sp = tS.p + m.normal * r;
    V3<S> wc = (sp + bp) * ADL(S, 0.5f);
    m.anchorA[0] = toLocal(wc, tS);
    m.anchorB[0] = toLocal(wc, tB);
    m.feature[0] = (kAdFeatSphereBox << 24) | region;
    return true;
}

// overlapOnAxis (sat.cpp:45-62)
template <class S>
AD_HD bool satAxis(const M3<S> &rA, const V3<S> &heA, const M3<S> &rB, const V3<S> &heB, const V3<S> &cd,
                   const V3<S> &axis, V3<S> &bestAxis, S &bestDepth) {
    S lsq = dot(axis, axis);
    if (val(lsq) < 1e-8f) return true;
    V3<S> na = axis * (ADL(S, 1.0f) / ssqrt(lsq));
    S distance = sabs(dot(cd, na));
    S d = (boxProjectedRadius(heA, rA, na) + boxProjectedRadius(heB, rB, na)) - distance;
    if (val(d) < 0.0f) return false;
    if (val(d) < val(bestDepth)) {
        bestDepth = d;
        bestAxis = na;
    }
    return true;
}

// testOBBOBB (sat.cpp:66-102)
template <class S>
AD_HDN bool satBoxBox(const V3<S> &heA, const Tf<S> &tA, const M3<S> &rA, const V3<S> &heB, const Tf<S> &tB,
                     const M3<S> &rB, V3<S> &axis, S &depth) {
    depth = ADL(S, 3.402823466e+38f);
    V3<S> cd = tB.p - tA.p;
    V3<S> ax[3] = {{rA.m00, rA.m10, rA.m20}, {rA.m01, rA.m11, rA.m21}, {rA.m02, rA.m12, rA.m22}};
    V3<S> bx[3] = {{rB.m00, rB.m10, rB.m20}, {rB.m01, rB.m11, rB.m21}, {rB.m02, rB.m12, rB.m22}};
    for (int i = 0; i < 3; ++i)
        if (!satAxis(rA, heA, rB, heB, cd, ax[i], axis, depth)) return false;
    for (int i = 0; i < 3; ++i)
        if (!satAxis(rA, heA, rB, heB, cd, bx[i], axis, depth)) return false;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            if (!satAxis(rA, heA, rB, heB, cd, cross(ax[i], bx[j]), axis, depth)) return false;
    return true;
}

// addFaceCandidates (narrowphase.cpp:281-304) for one source box face.
template <class S>
AD_HDN void boxFaceCandidates(const V3<S> &srcHe, const Tf<S> &srcTf, const V3<S> &othHe, const Tf<S> &othTf,
                             const V3<S> &dir, uint32_t source, V3<S> *contacts, S *depths, uint32_t *feats,
                             uint32_t &count) {
    S otherSurface = dot(boxSupport(othHe, othTf, -dir), dir);
    V3<S> ld = rotate(conj(srcTf.q), dir);
    int faceAxis = 0;
    float largest = sabs(val(ld.x));
    if (sabs(val(ld.y)) > largest) { faceAxis = 1; largest = sabs(val(ld.y)); }
    if (sabs(val(ld.z)) > largest) faceAxis = 2;
    const S comp = faceAxis == 0 ? ld.x : faceAxis == 1 ? ld.y : ld.z;
    const S one = ADL(S, 1.0f);
    S faceSign = val(comp) >= 0.0f ? one : -one;
    uint32_t signBit = val(comp) >= 0.0f ? 0u : 1u;
    S ext[3] = {srcHe.x, srcHe.y, srcHe.z};
    int fa = (faceAxis + 1) % 3, sa = (faceAxis + 2) % 3;
    Q<S> cq = conj(othTf.q);
    for (uint32_t vi = 0; vi < 4; ++vi) {
        S c[3] = {ADL(S, 0.0f), ADL(S, 0.0f), ADL(S, 0.0f)};
        c[faceAxis] = faceSign * ext[faceAxis];
        c[fa] = (vi & 1) ? ext[fa] : -ext[fa];
        c[sa] = (vi & 2) ? ext[sa] : -ext[sa];
        V3<S> v = toWorld(V3<S>{c[0], c[1], c[2]}, srcTf);
        V3<S> l = rotate(cq, v - othTf.p);
        const float tol = 1e-4f;
        if (!(sabs(val(l.x)) <= val(othHe.x) + tol && sabs(val(l.y)) <= val(othHe.y) + tol &&
              sabs(val(l.z)) <= val(othHe.z) + tol))
            continue;
        S depth = smax(dot(v, dir) - otherSurface, ADL(S, 0.0f));
        V3<S> cand = v - dir * (depth * ADL(S, 0.5f));
        if (count >= 4) continue;
        bool dup = false;
        for (uint32_t k = 0; k < count; ++k) {
            V3<S> dd = contacts[k] - cand;
            if (val(dot(dd, dd)) <= 1e-6f) dup = true;
        }
        if (dup) continue;
        depths[count] = depth;
        feats[count] = (kAdFeatBoxFace << 24) | (source << 16) | ((uint32_t)faceAxis << 8) | (signBit << 4) | vi;
        contacts[count++] = cand;
    }
}

// intersectBoxBox (narrowphase.cpp:250-324)
template <class S>
AD_HDN bool boxBox(const V3<S> &heA, const Tf<S> &tA, const V3<S> &heB, const Tf<S> &tB, Contact<S> &m) {
    M3<S> rA = toMat3(tA.q), rB = toMat3(tB.q);
    V3<S> normal;
    S penetration;
    if (!satBoxBox(heA, tA, rA, heB, tB, rB, normal, penetration)) return false;
    V3<S> cd = tB.p - tA.p;
    if (val(dot(cd, normal)) < 0.0f) normal = -normal;
    m.normal = normal;
    V3<S> contacts[4];
    S depths[4];
    uint32_t feats[4];
    uint32_t count = 0;
    boxFaceCandidates(heA, tA, heB, tB, normal, 0, contacts, depths, feats, count);
    boxFaceCandidates(heB, tB, heA, tA, -normal, 1, contacts, depths, feats, count);
    if (count == 0) {
        V3<S> tref = sabs(val(normal.x)) < 0.9f ? cst<S>(1.0f, 0.0f, 0.0f) : cst<S>(0.0f, 1.0f, 0.0f);
        V3<S> t1 = normalize(cross(normal, tref));
        V3<S> t2 = cross(normal, t1);
        S nc = (dot(tA.p, normal) + boxProjectedRadius(heA, rA, normal) + dot(tB.p, normal) -
                boxProjectedRadius(heB, rB, normal)) *
               ADL(S, 0.5f);
        auto mid = [&](const V3<S> &ax) {
            S cA = dot(tA.p, ax), cB = dot(tB.p, ax);
            S ra = boxProjectedRadius(heA, rA, ax), rb = boxProjectedRadius(heB, rB, ax);
            S lower = smax(cA - ra, cB - rb);
            S upper = smin(cA + ra, cB + rb);
            return (lower + upper) * ADL(S, 0.5f);
        };
        contacts[0] = normal * nc + t1 * mid(t1) + t2 * mid(t2);
        depths[0] = penetration;
        feats[0] = kAdFeatBoxFallback << 24;
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

// Shape dispatch with the box-sphere swap (narrowphase.cpp:326-374).
// shape: 0 sphere (dims.x = radius), 1 box (dims = half extents).
template <class S>
AD_HDN bool contactPair(uint32_t sa, const V3<S> &da, const Tf<S> &tA, uint32_t sb, const V3<S> &db,
                       const Tf<S> &tB, Contact<S> &m) {
    m.count = 0;
    bool hit;
    if (sa == 0 && sb == 0) {
        hit = sphereSphere(da.x, tA, db.x, tB, m);
    } else if (sa == 0) {
        hit = sphereBox(da.x, tA, db, tB, m);
    } else if (sb == 0) {
        hit = sphereBox(db.x, tB, da, tA, m);
        if (hit) {
            m.normal = -m.normal;
            for (uint32_t k = 0; k < m.count; ++k) {
                V3<S> t = m.anchorA[k];
                m.anchorA[k] = m.anchorB[k];
                m.anchorB[k] = t;
            }
        }
    } else {
        hit = boxBox(da, tA, db, tB, m);
    }
    return hit;
}

// --------------------------------------------------------------- prepare ---
// prepareContactPoints for one point (sequential_impulse_solver.cpp:101-214):
// the constants the velocity iterations use.
template <class S> struct Prepared {
    V3<S> offA, offB, t1, t2;
    S iem, bias, rv, itm00, itm01, itm11;
    V3<S> nrA, nrB, trA1, trB1, trA2, trB2;
    S ntr1, ntr2;
    bool tangentValid;
};
constexpr int kPreparedScalars = 38;

template <class S>
AD_HDN void preparePoint(const V3<S> &n, const V3<S> &anchorA, const V3<S> &anchorB, const S &penetration,
                        const Q<S> &qA, const Q<S> &qB, const M3<S> &IA, const M3<S> &IB, const S &imA,
                        const S &imB, const V3<S> &linA, const V3<S> &angA, const V3<S> &linB, const V3<S> &angB,
                        const S &rest, const S &inverseDt, Prepared<S> &o) {
    const S z = ADL(S, 0.0f);
    const V3<S> zv{z, z, z};
    o.offA = rotate(qA, anchorA);
    o.offB = rotate(qB, anchorB);
    o.t1 = o.t2 = o.nrA = o.nrB = o.trA1 = o.trB1 = o.trA2 = o.trB2 = zv;
    o.iem = o.bias = o.rv = o.itm00 = o.itm01 = o.itm11 = o.ntr1 = o.ntr2 = z;
    V3<S> tref = sabs(val(n.x)) < 0.9f ? cst<S>(1.0f, 0.0f, 0.0f) : cst<S>(0.0f, 1.0f, 0.0f);
    V3<S> t1 = cross(n, tref);
    S tl = ssqrt(dot(t1, t1));
    o.tangentValid = val(tl) > 1e-6f;
    if (!o.tangentValid) return;
    t1 = t1 / tl;
    V3<S> t2 = cross(n, t1);
    V3<S> vA = linA + cross(angA, o.offA), vB = linB + cross(angB, o.offB);
    S vin = dot(vB - vA, n);
    V3<S> jA = cross(o.offA, n), jB = cross(o.offB, n);
    V3<S> nrA = mul(IA, jA), nrB = mul(IB, jB);
    S ims = imA + imB;
    S iem = ims + dot(jA, nrA) + dot(jB, nrB);
    V3<S> tjA = cross(o.offA, t1), tjB = cross(o.offB, t1);
    V3<S> trA1 = mul(IA, tjA), trB1 = mul(IB, tjB);
    S tm00 = ims + dot(tjA, trA1) + dot(tjB, trB1);
    S ntr1 = ims * dot(n, t1) + dot(tjA, nrA) + dot(tjB, nrB);
    tjA = cross(o.offA, t2);
    tjB = cross(o.offB, t2);
    V3<S> trA2 = mul(IA, tjA), trB2 = mul(IB, tjB);
    S tm11 = ims + dot(tjA, trA2) + dot(tjB, trB2);
    S ntr2 = ims * dot(n, t2) + dot(tjA, nrA) + dot(tjB, nrB);
    S tm01 = dot(tjA, trA1) + dot(tjB, trB1);
    S det = tm00 * tm11 - tm01 * tm01;
    S itm00 = z, itm01 = z, itm11 = z;
    if (val(det) > 0.0f) {
        S inv = ADL(S, 1.0f) / det;
        itm00 = tm11 * inv;
        itm01 = -tm01 * inv;
        itm11 = tm00 * inv;
    }
    S bias = z, rv = z;
    if (!(val(iem) <= 0.0f)) {
        bias = smax(penetration - ADL(S, 0.005f), z) * (ADL(S, 0.2f) * inverseDt);
        rv = val(vin) < -1.0f ? rest * vin : z;
    }
    o.t1 = t1;
    o.t2 = t2;
    o.iem = iem;
    o.bias = bias;
    o.rv = rv;
    o.itm00 = itm00;
    o.itm01 = itm01;
    o.itm11 = itm11;
    o.nrA = nrA;
    o.nrB = nrB;
    o.trA1 = trA1;
    o.trB1 = trB1;
    o.trA2 = trA2;
    o.trB2 = trB2;
    o.ntr1 = ntr1;
    o.ntr2 = ntr2;
}

// Flat order of the prepared constants (index -> field).
template <class S> AD_HD void preparedPack(const Prepared<S> &o, S *out) {
    const V3<S> *vs[10] = {&o.offA, &o.offB, &o.t1, &o.t2, &o.nrA, &o.nrB, &o.trA1, &o.trB1, &o.trA2, &o.trB2};
    for (int i = 0; i < 10; ++i) {
        out[3 * i] = vs[i]->x;
        out[3 * i + 1] = vs[i]->y;
        out[3 * i + 2] = vs[i]->z;
    }
    out[30] = o.iem;
    out[31] = o.bias;
    out[32] = o.rv;
    out[33] = o.itm00;
    out[34] = o.itm01;
    out[35] = o.itm11;
    out[36] = o.ntr1;
    out[37] = o.ntr2;
}
template <class S> AD_HD V3<S> pv(const S *p, int i) { return {p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }
enum : int {
    kPOffA = 0, kPOffB = 1, kPT1 = 2, kPT2 = 3, kPNrA = 4, kPNrB = 5, kPTrA1 = 6, kPTrB1 = 7, kPTrA2 = 8, kPTrB2 = 9,
    kPIem = 30, kPBias = 31, kPRv = 32, kPItm00 = 33, kPItm01 = 34, kPItm11 = 35, kPNtr1 = 36, kPNtr2 = 37
};

} // namespace ad
} // namespace pe
