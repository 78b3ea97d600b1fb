// FP64 CPU evaluation of the differentiable rollout (include/phys_gb300_fp64.h):
// the scalar-generic step and adjoint of ad_world.cuh instantiated for double
// on one host thread.  Every step's start state, cache and scratch are kept, so
// no recomputation is needed.
#include <cstring>
#include <string>
#include <vector>

#include "ad_world.cuh"
#include "phys_gb300_fp64.h"

namespace {

using namespace pe::ad;
using S = double;

void setErr(char *err, int len, const std::string &msg) {
    if (err && len > 0) {
        std::strncpy(err, msg.c_str(), (size_t)len - 1);
        err[len - 1] = 0;
    }
}

struct StateMem {
    std::vector<S> x, q, v, w;
    explicit StateMem(uint32_t n = 0) : x(3 * n), q(4 * n), v(3 * n), w(3 * n) {}
    StateView<S> view() { return {x.data(), q.data(), v.data(), w.data()}; }
};

struct CacheMem {
    uint32_t count = 0;
    std::vector<unsigned long long> key;
    std::vector<S> anchorA, anchorB, lam;
    explicit CacheMem(uint32_t cap = 0) : key(cap), anchorA(3 * cap), anchorB(3 * cap), lam(3 * cap) {}
    CacheView<S> view() {
        return {&count, key.data(), anchorA.data(), anchorB.data(), lam.data(), (uint32_t)key.size()};
    }
};

struct ScratchMem {
    std::vector<S> aabb, mNormal, mMu, mRest, mAnchorA, mAnchorB, mDepth, pp, pm, lam, lamInit, tape;
    std::vector<uint32_t> pairA, pairB, mA, mB, mCount, mFeature, color, order, colorStart, cacheSrc, counts;
    std::vector<unsigned long long> sortKeys, bodyUsed, bpEntries, bpPairs;
    std::vector<int32_t> match;
    ScratchMem(uint32_t n, uint32_t maxPairs, uint32_t maxM, int iterations)
        : aabb(6 * n), mNormal(3 * maxM), mMu(maxM), mRest(maxM), mAnchorA(12 * maxM), mAnchorB(12 * maxM),
          mDepth(4 * maxM), pp((size_t)4 * maxM * kPreparedScalars), pm((size_t)maxM * kPmScalars), lam(12 * maxM),
          lamInit(12 * maxM), tape((size_t)(iterations > 0 ? iterations : 1) * maxM * kTapeScalars), pairA(maxPairs),
          pairB(maxPairs), mA(maxM), mB(maxM), mCount(maxM), mFeature(4 * maxM), color(maxM), order(maxM),
          colorStart(maxM + 1), cacheSrc(4 * maxM), counts(4), sortKeys(maxM), bodyUsed(2 * n),
          bpEntries(nextPow2u(n > 0 ? n : 1)), bpPairs(nextPow2u(maxPairs > 0 ? maxPairs : 1)), match(4 * maxM) {}
    StepScratch<S> view() {
        StepScratch<S> s;
        s.aabb = aabb.data();
        s.pairA = pairA.data();
        s.pairB = pairB.data();
        s.mA = mA.data();
        s.mB = mB.data();
        s.mCount = mCount.data();
        s.mFeature = mFeature.data();
        s.mNormal = mNormal.data();
        s.mMu = mMu.data();
        s.mRest = mRest.data();
        s.mAnchorA = mAnchorA.data();
        s.mAnchorB = mAnchorB.data();
        s.mDepth = mDepth.data();
        s.color = color.data();
        s.order = order.data();
        s.sortKeys = sortKeys.data();
        s.bodyUsed = bodyUsed.data();
        s.colorStart = colorStart.data();
        s.pp = pp.data();
        s.pm = pm.data();
        s.lam = lam.data();
        s.lamInit = lamInit.data();
        s.match = match.data();
        s.tape = tape.data();
        s.cacheSrc = cacheSrc.data();
        s.counts = counts.data();
        s.bpEntries = bpEntries.data();
        s.bpPairs = bpPairs.data();
        return s;
    }
};

const char *errorText(uint32_t bits) {
    if (bits & kAdErrPairs) return "candidate pairs exceed the rollout's pair capacity";
    if (bits & kAdErrManifolds) return "contact manifolds exceed the rollout's manifold capacity";
    if (bits & kAdErrColors) return "more than 128 solver colours";
    if (bits & kAdErrCache) return "warm-start cache overflow";
    if (bits & kAdErrReplay) return "the adjoint's replay of a contact differed from the forward pass";
    return "rollout failed";
}

} // namespace

extern "C" {

int pe_fp64_body_properties(int shape, const float *dims, float density, int is_static, float *mass,
                            float *inv_inertia, char *err, int err_len) {
    // RigidBody::createSphere / createBox (src/dynamics/rigid_body.cpp:25-91)
    const float pi = 3.14159265358979323846f;
    const float minSize = 0.01f * 0.01f, maxSize = 64.0f * 64.0f;
    float volume;
    if (shape == 0) {
        const float r = dims[0];
        volume = (4.0f / 3.0f) * pi * r * r * r;
        if (volume < minSize || volume > maxSize) return setErr(err, err_len, "sphere size out of range"), 1;
    } else {
        if (dims[0] <= 0.0f || dims[1] <= 0.0f || dims[2] <= 0.0f)
            return setErr(err, err_len, "Box dimensions must be positive"), 1;
        volume = dims[0] * dims[1] * dims[2];
        if (volume < minSize || volume > maxSize) return setErr(err, err_len, "box size out of range"), 1;
    }
    if (!(density >= 0.2f && density <= 21.4f)) return setErr(err, err_len, "Density is out of range"), 1;
    const float m = volume * density;
    *mass = m;
    inv_inertia[0] = inv_inertia[1] = inv_inertia[2] = 0.0f;
    if (!is_static) {
        if (shape == 0) {
            const float r = dims[0];
            if (m > 0.0f && r > 0.0f) inv_inertia[0] = inv_inertia[1] = inv_inertia[2] = 1.0f / (0.4f * m * r * r);
        } else if (m > 0.0f) {
            const float w = dims[0], h = dims[1], d = dims[2];
            const float factor = 12.0f / m;
            inv_inertia[0] = factor / (h * h + d * d);
            inv_inertia[1] = factor / (w * w + d * d);
            inv_inertia[2] = factor / (w * w + h * h);
        }
    }
    return 0;
}

int pe_fp64_rollout(uint32_t n, const uint8_t *shape, const uint8_t *is_static, const double *half_extents,
                    const double *inv_inertia, const double *gravity, double dt, int iterations, uint32_t steps,
                    const double *x0, const double *q0, const double *v0, const double *w0, const double *mass,
                    const double *friction, const double *restitution, double *x_final, double *q_final,
                    double *v_final, double *w_final, const double *d_final_x, const double *d_final_q,
                    const double *d_final_v, const double *d_final_w, double *d_x0, double *d_q0, double *d_v0,
                    double *d_w0, double *d_mass, double *d_friction, double *d_restitution, char *err,
                    int err_len) {
    if (n == 0 || n > 4096 || !shape || !is_static || !half_extents || !inv_inertia || !gravity || !x0 || !q0 ||
        !v0 || !w0 || !mass || !friction || !restitution || iterations < 0)
        return setErr(err, err_len, "invalid arguments"), 1;
    const uint32_t maxPairs = 64 * n + 256;
    const uint32_t maxM = nextPow2u(8 * n + 64);
    WorldParams<S> W;
    W.n = n;
    W.shape = shape;
    W.isStatic = is_static;
    W.dims = half_extents;
    W.iinv = inv_inertia;
    W.mass = mass;
    W.mu = friction;
    W.rest = restitution;
    W.gx = gravity[0];
    W.gy = gravity[1];
    W.gz = gravity[2];
    W.dt = dt;
    W.iterations = iterations;
    W.maxPairs = maxPairs;
    W.maxManifolds = maxM;
    std::vector<StateMem> state(steps + 1, StateMem(n));
    std::vector<CacheMem> cache(steps + 1, CacheMem(4 * maxM));
    std::vector<ScratchMem> scratch;
    scratch.reserve(steps);
    std::memcpy(state[0].x.data(), x0, 3 * n * sizeof(S));
    std::memcpy(state[0].q.data(), q0, 4 * n * sizeof(S));
    std::memcpy(state[0].v.data(), v0, 3 * n * sizeof(S));
    std::memcpy(state[0].w.data(), w0, 3 * n * sizeof(S));
    for (uint32_t t = 0; t < steps; ++t) {
        scratch.emplace_back(n, maxPairs, maxM, iterations);
        StateView<S> in = state[t].view();
        CacheView<S> cin = cache[t].view();
        forwardStep<S, HostTeam>(W, in, cin, state[t + 1].view(), cache[t + 1].view(), scratch[t].view(), true);
        if (scratch[t].counts[3]) return setErr(err, err_len, errorText(scratch[t].counts[3])), 2;
    }
    const StateMem &fin = state[steps];
    if (x_final) std::memcpy(x_final, fin.x.data(), 3 * n * sizeof(S));
    if (q_final) std::memcpy(q_final, fin.q.data(), 4 * n * sizeof(S));
    if (v_final) std::memcpy(v_final, fin.v.data(), 3 * n * sizeof(S));
    if (w_final) std::memcpy(w_final, fin.w.data(), 3 * n * sizeof(S));
    if (!d_final_x && !d_final_q && !d_final_v && !d_final_w) return 0;

    std::vector<S> ax(3 * n, 0.0), aq(4 * n, 0.0), av(3 * n, 0.0), aw(3 * n, 0.0);
    if (d_final_x) std::memcpy(ax.data(), d_final_x, 3 * n * sizeof(S));
    if (d_final_q) std::memcpy(aq.data(), d_final_q, 4 * n * sizeof(S));
    if (d_final_v) std::memcpy(av.data(), d_final_v, 3 * n * sizeof(S));
    if (d_final_w) std::memcpy(aw.data(), d_final_w, 3 * n * sizeof(S));
    std::vector<S> alam(12 * maxM, 0.0), app((size_t)4 * maxM * kPreparedScalars), apm((size_t)maxM * kPmScalars),
        an(3 * maxM), amuM(maxM), arestM(maxM), acache(12 * maxM), amass(n, 0.0), amu(n, 0.0), arest(n, 0.0);
    std::vector<S> v1v(3 * n), v1w(3 * n);
    AdjointView<S> adj{ax.data(),    aq.data(),    av.data(),   aw.data(),     alam.data(),
                       app.data(),   apm.data(),   an.data(),   amuM.data(),   arestM.data(),
                       acache.data(), amass.data(), amu.data(), arest.data()};
    for (int t = (int)steps - 1; t >= 0; --t) {
        StateView<S> v1{nullptr, nullptr, v1v.data(), v1w.data()};
        backwardStep<S, HostTeam>(W, state[t].view(), cache[t].view(), state[t + 1].view(), v1, scratch[t].view(),
                                  adj);
        if (scratch[t].counts[3]) return setErr(err, err_len, errorText(scratch[t].counts[3])), 3;
        // adjoint of this step's input cache -> adjoint of the previous step's final impulses
        std::fill(alam.begin(), alam.end(), 0.0);
        if (t > 0) {
            const uint32_t cnt = cache[t].count;
            for (uint32_t e = 0; e < cnt; ++e) {
                const uint32_t kp = scratch[t - 1].cacheSrc[e];
                for (int j = 0; j < 3; ++j) alam[3 * kp + j] += acache[3 * e + j];
            }
        }
    }
    if (d_x0) std::memcpy(d_x0, ax.data(), 3 * n * sizeof(S));
    if (d_q0) std::memcpy(d_q0, aq.data(), 4 * n * sizeof(S));
    if (d_v0) std::memcpy(d_v0, av.data(), 3 * n * sizeof(S));
    if (d_w0) std::memcpy(d_w0, aw.data(), 3 * n * sizeof(S));
    if (d_mass) std::memcpy(d_mass, amass.data(), n * sizeof(S));
    if (d_friction) std::memcpy(d_friction, amu.data(), n * sizeof(S));
    if (d_restitution) std::memcpy(d_restitution, arest.data(), n * sizeof(S));
    return 0;
}

} // extern "C"
