// Per-body and per-collider stages of the step.
//   k_integrate_aabb : RigidBody::integrateVelocity (src/dynamics/rigid_body.cpp:94-101)
//                      fused with Aabb::fromCollider (src/collision/aabb.cpp:8-32) and
//                      the SAP sort-key build (src/collision/broadphase.cpp:205-217).
//   k_collect        : gather of live colliders for the broadphase
//                      (src/world/physics_world.cpp:570-581) when slots have holes.
//   k_integrate_pose : integratePosition / integrateRotation
//                      (src/dynamics/rigid_body.cpp:103-125, physics_world.cpp:759-767).
#include "pe_bodies.cuh"
#include "pe_kernels.cuh"
#include "pe_stages.h"

namespace pe {

// One body (velocity) and one collider (AABB, SAP key) of k_integrate_aabb.
__device__ __forceinline__ void integrateAabbOne(const WorldView &w, uint32_t *sapKeys, uint32_t *sapVals, uint32_t i) {
    if (i < w.nb) {
        const uint32_t f = w.bflags[i];
        V3 lin = f4xyz(w.cur.lin[i]);
        bool integrate = (f & kBodyAlive) && !(f & kBodyStatic);
        if (w.sleepMode) {
            // integrateVelocity skips sleeping bodies; SleepState::integratedVelocity
            // = !isSleeping() (physics_world.cpp:528-537); the island scratch
            // of this step starts empty.
            const uint32_t sf = w.sleepIn[i];
            const bool asleep = (sf & kSleepAsleep) != 0;
            if (asleep) integrate = false;
            w.sleepOut[i] = (sf & ~kSleepIntegrated) | (asleep && !(f & kBodyStatic) ? 0u : kSleepIntegrated);
            w.quietOut[i] = w.quietIn[i];
            w.sleepParent[i] = i;
            w.sleepIsland[i] = 0u;
            w.sleepQuietMin[i] = 0x7F800000u;  // +inf: no quiet time folded in yet
        }
        if (integrate) {
            const float *force3 = w.io ? w.io->force3 : w.force3;
            const uint32_t force3n = w.io ? w.io->force3n : w.force3n;
            const V3 force = force3 ? (i < force3n ? V3{force3[3 * i], force3[3 * i + 1], force3[3 * i + 2]}
                                                   : V3{0.0f, 0.0f, 0.0f})
                             : w.force ? f4xyz(w.force[i]) : V3{0.0f, 0.0f, 0.0f};
            lin = integrateVelocity(lin, V3{w.gx, w.gy, w.gz}, force, w.mat[i].x, w.dt);
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
        if (w.npRec) {
            const float4 s = w.cshape[i], m = w.mat[b];
            float4 *r = w.npRec + 4 * (size_t)i;
            r[0] = make_float4(t.p.x, t.p.y, t.p.z, s.x);
            r[1] = make_float4(t.q.x, t.q.y, t.q.z, t.q.w);
            r[2] = make_float4(s.y, s.z, s.w, __uint_as_float(cf));
            r[3] = make_float4(m.y, m.z, __uint_as_float(b), __uint_as_float(w.cbgen[i]));
        }
        if (sapKeys) {
            sapKeys[i] = orderedFloatKey(mn.x);
            if (sapVals) sapVals[i] = i;
        }
    }
}

// st (nullable): the step's counters are initialised here as well, which saves
// a launch at the head of the step; so is clearing `fill` (nFill words set to
// all ones: the hashed grid's empty bucket lists), which saves a memset node.
__global__ void k_integrate_aabb(WorldView w, uint32_t *sapKeys, uint32_t *sapVals, DevStats *st,
                                 uint32_t inputCount, uint32_t *fill, uint32_t nFill) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (st && i == 0) {
        initStepStats(st, inputCount);
        st->stamp[0] = globalNs();
    }
    for (uint32_t j = i; j < nFill; j += gridDim.x * blockDim.x) fill[j] = 0xFFFFFFFFu;
    integrateAabbOne(w, sapKeys, sapVals, i);
    if (st) {
        __syncthreads();
        if (threadIdx.x == 0) atomicMax(&st->stamp[1], globalNs());
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

// hostOut (nullable, host memory the device can write): the last block to
// finish copies the step's counters there, which saves a copy node after the
// kernel; done is its arrival counter (left at zero for the next step).
__global__ void k_integrate_pose(WorldView w, DevStats *st, DevStats *hostOut, uint32_t *done) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (st && i == 0) st->stamp[4] = globalNs();
    if (i < w.nb) {
        const uint32_t f = w.bflags[i];
        float4 p4 = w.cur.pos[i], q4 = w.cur.rot[i];
        const bool dyn = (f & kBodyAlive) && !(f & kBodyStatic);
        const uint32_t sf = w.sleepMode ? w.sleepOut[i] : 0u;
        if (dyn && !(sf & kSleepAsleep)) {
            V3 pos = f4xyz(p4);
            Q rot = f4q(q4);
            integratePose(pos, rot, f4xyz(w.nxt.lin[i]), f4xyz(w.nxt.ang[i]), w.dt);
            p4 = make4(pos, 0.0f);
            q4 = make4(rot);
        }
        w.nxt.pos[i] = p4;
        w.nxt.rot[i] = q4;
        float *pos3 = w.io ? w.io->pos3 : w.pos3;
        if (pos3) {
            pos3[3 * i] = p4.x;
            pos3[3 * i + 1] = p4.y;
            pos3[3 * i + 2] = p4.z;
        }
        if (w.io && w.io->rot4) w.io->rot4[i] = q4;
        if (w.sleepMode && dyn) {
            // finishSleeping's first loop (physics_world.cpp:474-490): the quiet
            // time of an awake body, folded into its island's minimum.
            const float quietSpeedSquared = 0.05f * 0.05f, timeToSleep = 0.5f;
            float q = w.quietOut[i];
            if (!(sf & kSleepAsleep)) {
                const V3 v = f4xyz(w.nxt.lin[i]), a = f4xyz(w.nxt.ang[i]);
                if (!(sf & kSleepWake) && w.dt > 0.0f && isfinite(w.dt) && dot(v, v) <= quietSpeedSquared &&
                    dot(a, a) <= quietSpeedSquared) {
                    const float t = q + w.dt;
                    q = timeToSleep < t ? timeToSleep : t;
                } else {
                    q = 0.0f;
                }
                w.quietOut[i] = q;
            }
            atomicMin(&w.sleepQuietMin[w.sleepParent[i]], __float_as_uint(q));
        }
    }
    if (st) {
        __syncthreads();
        __shared__ bool s_last;
        if (threadIdx.x == 0) {
            atomicMax(&st->stamp[5], globalNs());
            s_last = false;
            if (hostOut) {
                __threadfence();
                s_last = atomicAdd(done, 1u) == gridDim.x - 1;
            }
        }
        __syncthreads();
        if (s_last) {
            // every block's counters are in: copy them out (8 bytes per lane)
            __threadfence();
            const unsigned long long *src = reinterpret_cast<const unsigned long long *>(st);
            unsigned long long *dst = reinterpret_cast<unsigned long long *>(hostOut);
            for (uint32_t k = threadIdx.x; k < sizeof(DevStats) / 8; k += blockDim.x) dst[k] = __ldcg(&src[k]);
            if (threadIdx.x == 0) *done = 0;
        }
    }
}

// Caller forces (3 floats per body) into the force array; RigidBody::applyForce
// ignores static bodies (rigid_body.cpp), dead slots get none.
__global__ void k_expand_forces(const float *f3, const uint32_t *bflags, float4 *force, uint32_t n, uint32_t *sleep) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t fl = bflags[i];
    const bool dyn = (fl & kBodyAlive) && !(fl & kBodyStatic);
    const float fx = f3[3 * i], fy = f3[3 * i + 1], fz = f3[3 * i + 2];
    force[i] = dyn ? make_float4(fx, fy, fz, 0.0f) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (sleep && dyn && (fx != 0.0f || fy != 0.0f || fz != 0.0f)) sleep[i] = (sleep[i] & ~kSleepAsleep) | kSleepWake;
}

// Positions as 3 floats per body (the caller's layout).
__global__ void k_pack_positions(const float4 *pos, float *p3, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    p3[3 * i] = p.x;
    p3[3 * i + 1] = p.y;
    p3[3 * i + 2] = p.z;
}

void launchExpandForces(const float *f3, const uint32_t *bflags, float4 *force, uint32_t n, cudaStream_t s,
                        uint32_t *sleep) {
    if (!n) return;
    k_expand_forces<<<(n + 255) / 256, 256, 0, s>>>(f3, bflags, force, n, sleep);
    PE_LAUNCHED();
}

void launchPackPositions(const float4 *pos, float *p3, uint32_t n, cudaStream_t s) {
    if (!n) return;
    k_pack_positions<<<(n + 255) / 256, 256, 0, s>>>(pos, p3, n);
    PE_LAUNCHED();
}

void launchIntegrateAabb(const WorldView &w, uint32_t *sapKeys, uint32_t *sapVals, DevStats *st,
                         uint32_t inputCount, cudaStream_t s, uint32_t *fill, uint32_t nFill) {
    uint32_t n = w.nb > w.nc ? w.nb : w.nc;
    if (!n) {
        if (st) launchStepInit(st, inputCount, s);
        if (nFill) PE_CHECK(cudaMemsetAsync(fill, 0xFF, nFill * sizeof(uint32_t), s));
        return;
    }
    k_integrate_aabb<<<(n + 255) / 256, 256, 0, s>>>(w, sapKeys, sapVals, st, inputCount, fill, nFill);
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

void launchIntegratePose(const WorldView &w, cudaStream_t s, DevStats *st, DevStats *hostOut, uint32_t *done) {
    if (!w.nb) return;
    k_integrate_pose<<<(w.nb + 255) / 256, 256, 0, s>>>(w, st, hostOut, done);
    PE_LAUNCHED();
}

} // namespace pe
