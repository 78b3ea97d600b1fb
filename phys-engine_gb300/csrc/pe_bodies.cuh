// Per-body / per-collider device helpers shared by the single-world kernels and
// the batched-world kernel: collider world transform (physics_world.cpp:658-667)
// and Aabb::fromCollider (src/collision/aabb.cpp:8-32), plus the two body
// integrators (src/dynamics/rigid_body.cpp:94-125).
#pragma once
#include "pe_engine.h"
#include "pe_math.cuh"

namespace pe {

__device__ __forceinline__ Tf colliderWorld(const WorldView &w, uint32_t c, const V3 &bp, const Q &bq) {
    V3 lp = w.clpos ? f4xyz(w.clpos[c]) : V3{0.0f, 0.0f, 0.0f};
    Q lq = w.clrot ? f4q(w.clrot[c]) : qidentity();
    return Tf{bp + rotate(bq, lp), qmul(bq, lq)};
}

__device__ __forceinline__ void colliderAabb(const WorldView &w, uint32_t c, const Tf &t, V3 &mn, V3 &mx) {
    const uint32_t shape = colliderShape(w.cflags[c]);
    const float4 s = w.cshape[c];
    if (shape == kShapeSphere) {
        V3 r{s.x, s.x, s.x};
        mn = t.p - r;
        mx = t.p + r;
        return;
    }
    if (shape == kShapeHull) {
        const uint32_t h = __float_as_uint(s.w);
        const uint32_t b = w.hullOffset[h], e = w.hullOffset[h + 1];
        for (uint32_t k = b; k < e; ++k) {
            V3 v = toWorld(f4xyz(w.hullVerts[k]), t);
            if (k == b) {
                mn = v;
                mx = v;
            } else {
                mn = V3{smin(mn.x, v.x), smin(mn.y, v.y), smin(mn.z, v.z)};
                mx = V3{smax(mx.x, v.x), smax(mx.y, v.y), smax(mx.z, v.z)};
            }
        }
        return;
    }
    M3 m = toMat3(t.q);
    V3 e{fabsf(m.m00) * s.x + fabsf(m.m01) * s.y + fabsf(m.m02) * s.z,
         fabsf(m.m10) * s.x + fabsf(m.m11) * s.y + fabsf(m.m12) * s.z,
         fabsf(m.m20) * s.x + fabsf(m.m21) * s.y + fabsf(m.m22) * s.z};
    mn = t.p - e;
    mx = t.p + e;
}

// RigidBody::integrateVelocity: v += (g + F * invMass) * dt.
__device__ __forceinline__ V3 integrateVelocity(V3 lin, const V3 &g, const V3 &force, float invMass, float dt) {
    V3 acc = g + force * invMass;
    lin += acc * dt;
    return lin;
}

// RigidBody::integratePosition + integrateRotation.
__device__ __forceinline__ void integratePose(V3 &pos, Q &rot, const V3 &lin, const V3 &ang, float dt) {
    pos += lin * dt;
    Q spin{ang.x, ang.y, ang.z, 0.0f};
    Q d = qmul(spin, rot);
    const float h = 0.5f * dt;
    rot.x += h * d.x;
    rot.y += h * d.y;
    rot.z += h * d.z;
    rot.w += h * d.w;
    rot = qnormalized(rot);
}

} // namespace pe
