// Per-body and per-collider stages of the step.
//   k_integrate_aabb : RigidBody::integrateVelocity (src/dynamics/rigid_body.cpp:94-101)
//                      fused with Aabb::fromCollider (src/collision/aabb.cpp:8-32) and
//                      the SAP sort-key build (src/collision/broadphase.cpp:205-217).
//   k_collect        : gather of live colliders for the broadphase
//                      (src/world/physics_world.cpp:570-581) when slots have holes.
//   k_integrate_pose : integratePosition / integrateRotation
//                      (src/dynamics/rigid_body.cpp:103-125, physics_world.cpp:759-767).
#include "pe_kernels.cuh"

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

__global__ void k_integrate_aabb(WorldView w, uint32_t *sapKeys, uint32_t *sapVals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < w.nb) {
        const uint32_t f = w.bflags[i];
        V3 lin = f4xyz(w.cur.lin[i]);
        if ((f & kBodyAlive) && !(f & kBodyStatic)) {
            const float invMass = w.mat[i].x;
            V3 force = w.force ? f4xyz(w.force[i]) : V3{0.0f, 0.0f, 0.0f};
            V3 acc = V3{w.gx, w.gy, w.gz} + force * invMass;
            lin += acc * w.dt;
        }
        w.nxt.lin[i] = make4(lin, 0.0f);
        w.nxt.ang[i] = w.cur.ang[i];
    }
    if (i < w.nc) {
        const uint32_t cf = w.cflags[i];
        const uint32_t b = w.cbody[i];
        if (!(cf & kColliderAlive) || b >= w.nb || !(w.bflags[b] & kBodyAlive) || w.bgen[b] != w.cbgen[i]) return;
        Tf t = colliderWorld(w, i, f4xyz(w.cur.pos[b]), f4q(w.cur.rot[b]));
        V3 mn, mx;
        colliderAabb(w, i, t, mn, mx);
        w.aabbMin[i] = make4(mn, 0.0f);
        w.aabbMax[i] = make4(mx, 0.0f);
        if (sapKeys) {
            sapKeys[i] = orderedFloatKey(mn.x);
            sapVals[i] = i;
        }
    }
}

// Live-collider flags for the compaction of bounds (slot order is kept).
__global__ void k_collect_flags(WorldView w, uint32_t *flags) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nc) return;
    const uint32_t cf = w.cflags[i];
    const uint32_t b = w.cbody[i];
    flags[i] = ((cf & kColliderAlive) && b < w.nb && (w.bflags[b] & kBodyAlive) && w.bgen[b] == w.cbgen[i]) ? 1u : 0u;
}

__global__ void k_collect_scatter(WorldView w, const uint32_t *flags, const uint32_t *pos, float4 *inMin,
                                  float4 *inMax, uint32_t *inSlot, uint32_t *sapKeys, uint32_t *sapVals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nc || !flags[i]) return;
    const uint32_t k = pos[i];
    float4 mn = w.aabbMin[i];
    inMin[k] = mn;
    inMax[k] = w.aabbMax[i];
    inSlot[k] = i;
    if (sapKeys) {
        sapKeys[k] = orderedFloatKey(mn.x);
        sapVals[k] = k;
    }
}

__global__ void k_integrate_pose(WorldView w) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.nb) return;
    const uint32_t f = w.bflags[i];
    float4 p4 = w.cur.pos[i], q4 = w.cur.rot[i];
    if ((f & kBodyAlive) && !(f & kBodyStatic)) {
        V3 pos = f4xyz(p4);
        V3 lin = f4xyz(w.nxt.lin[i]);
        V3 ang = f4xyz(w.nxt.ang[i]);
        pos += lin * w.dt;
        Q rot = f4q(q4);
        Q spin{ang.x, ang.y, ang.z, 0.0f};
        Q d = qmul(spin, rot);
        const float h = 0.5f * w.dt;
        rot.x += h * d.x;
        rot.y += h * d.y;
        rot.z += h * d.z;
        rot.w += h * d.w;
        rot = qnormalized(rot);
        p4 = make4(pos, 0.0f);
        q4 = make4(rot);
    }
    w.nxt.pos[i] = p4;
    w.nxt.rot[i] = q4;
}

void launchIntegrateAabb(const WorldView &w, uint32_t *sapKeys, uint32_t *sapVals, cudaStream_t s) {
    uint32_t n = w.nb > w.nc ? w.nb : w.nc;
    if (!n) return;
    k_integrate_aabb<<<(n + 255) / 256, 256, 0, s>>>(w, sapKeys, sapVals);
    PE_LAUNCHED();
}

void launchCollect(const WorldView &w, uint32_t *flags, uint32_t *pos, float4 *inMin, float4 *inMax, uint32_t *inSlot,
                   uint32_t *sapKeys, uint32_t *sapVals, uint32_t *d_count, Scratch &ws, uint32_t *d_err,
                   cudaStream_t s) {
    if (!w.nc) return;
    k_collect_flags<<<(w.nc + 255) / 256, 256, 0, s>>>(w, flags);
    PE_LAUNCHED();
    launchScanExclusive(flags, pos, nullptr, w.nc, d_count, ws, d_err, s);
    k_collect_scatter<<<(w.nc + 255) / 256, 256, 0, s>>>(w, flags, pos, inMin, inMax, inSlot, sapKeys, sapVals);
    PE_LAUNCHED();
}

void launchIntegratePose(const WorldView &w, cudaStream_t s) {
    if (!w.nb) return;
    k_integrate_pose<<<(w.nb + 255) / 256, 256, 0, s>>>(w);
    PE_LAUNCHED();
}

} // namespace pe
