// GPU world: host mirror, device state and the step pipeline
// (PhysicsWorld::step, src/world/physics_world.cpp:518-782, with sleeping
// islands, :341-516).
#include "world.h"

#include <algorithm>
#include <cstring>

namespace pe {

namespace {
template <class T> void upload(DeviceArray<T> &d, const std::vector<T> &h, cudaStream_t s) {
    d.reserve(h.size());
    if (!h.empty()) PE_CHECK(cudaMemcpyAsync(d.ptr, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
}
// Grows d to at least n elements keeping its first `keep` elements.
template <class T> void reserveKeep(DeviceArray<T> &d, size_t n, size_t keep) {
    if (n <= d.count && d.ptr) return;
    DeviceArray<T> g;
    g.reserve(n);
    keep = std::min(keep, d.count);
    if (d.ptr && keep) PE_CHECK(cudaMemcpy(g.ptr, d.ptr, keep * sizeof(T), cudaMemcpyDeviceToDevice));
    d.swap(g);
}
inline uint32_t grow(uint32_t need, uint32_t have) {
    uint64_t n = std::max<uint64_t>(need, have);
    n = n + n / 2 + 1024;
    return (uint32_t)std::min<uint64_t>(n, 0xFFFFFFF0u);
}
} // namespace

World::World(int device) : device_(device) {
    PE_CHECK(cudaSetDevice(device_));
    PE_CHECK(cudaDeviceGetAttribute(&smCount_, cudaDevAttrMultiProcessorCount, device_));
    PE_CHECK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    PE_CHECK(cudaMallocHost(&hostStats_, sizeof(DevStats)));
    std::memset(hostStats_, 0, sizeof(DevStats));
    PE_CHECK(cudaHostAlloc(reinterpret_cast<void **>(&ioHost_), sizeof(StepIo), cudaHostAllocMapped));
    std::memset(ioHost_, 0, sizeof(StepIo));
    PE_CHECK(cudaHostGetDevicePointer(reinterpret_cast<void **>(&ioDev_), ioHost_, 0));
    stats_.reserve(1);
    poseDone_.reserve(1);
    cCount_.reserve(2);
    sEpoch_.reserve(1);
}

World::~World() {
    if (stream_) cudaStreamSynchronize(stream_);
    dropGraphs();
    if (hostStats_) cudaFreeHost(hostStats_);
    if (ioHost_) cudaFreeHost(ioHost_);
    if (pinned_) cudaFreeHost(pinned_);
    if (stream_) cudaStreamDestroy(stream_);
}

void World::syncDevice() { PE_CHECK(cudaStreamSynchronize(stream_)); }

void *World::deviceAddress(const void *p, size_t align) const { return pe::deviceAddress(p, align, device_); }

// ---------------------------------------------------------------- slots ----
uint32_t World::addBody(const HostBody &b, uint32_t &generation) {
    pull();
    hostDirty_ = true;
    if (!freeBodies.empty()) {
        uint32_t idx = freeBodies.back();
        freeBodies.pop_back();
        uint32_t g = bodies[idx].generation;
        bodies[idx] = b;
        bodies[idx].generation = g;
        bodies[idx].alive = true;
        bodies[idx].wakeUp();  // PhysicsWorld::addBody wakes the body (physics_world.cpp:171, :177)
        generation = g;
        return idx;
    }
    bodies.push_back(b);
    bodies.back().generation = 0;
    bodies.back().alive = true;
    bodies.back().wakeUp();
    generation = 0;
    return (uint32_t)bodies.size() - 1;
}

uint32_t World::addCollider(const HostCollider &c, uint32_t &generation) {
    pull();
    hostDirty_ = true;
    // PhysicsWorld::addCollider wakes the collider's body (physics_world.cpp:276-281)
    if (HostBody *b = body(c.body, c.bodyGeneration)) b->wakeUp();
    if (!freeColliders.empty()) {
        uint32_t idx = freeColliders.back();
        freeColliders.pop_back();
        uint32_t g = colliders[idx].generation;
        colliders[idx] = c;
        colliders[idx].generation = g;
        colliders[idx].alive = true;
        generation = g;
        return idx;
    }
    colliders.push_back(c);
    colliders.back().generation = 0;
    colliders.back().alive = true;
    generation = 0;
    return (uint32_t)colliders.size() - 1;
}

void World::removeBody(uint32_t index, uint32_t generation) {
    pull();
    if (index >= bodies.size()) return;
    HostBody &b = bodies[index];
    if (!b.alive || b.generation != generation) return;
    hostDirty_ = true;
    wakeContacts(index, generation);
    b.alive = false;
    b.generation++;
    freeBodies.push_back(index);
    for (uint32_t i = 0; i < colliders.size(); ++i) {
        HostCollider &c = colliders[i];
        if (c.alive && c.body == index && c.bodyGeneration == generation) {
            c.alive = false;
            c.generation++;
            freeColliders.push_back(i);
        }
    }
}

void World::removeCollider(uint32_t index, uint32_t generation) {
    pull();
    if (index >= colliders.size()) return;
    HostCollider &c = colliders[index];
    if (!c.alive || c.generation != generation) return;
    hostDirty_ = true;
    // PhysicsWorld::removeCollider wakes the body and its contacts (physics_world.cpp:309-311)
    if (HostBody *b = body(c.body, c.bodyGeneration)) b->wakeUp();
    wakeContacts(c.body, c.bodyGeneration);
    c.alive = false;
    c.generation++;
    freeColliders.push_back(index);
}

bool World::setCollider(uint32_t index, uint32_t generation, uint32_t bodyIndex, uint32_t bodyGeneration,
                        uint32_t shape, const float *dims, const float *lpos, const float *lrot) {
    pull();
    HostCollider *c = collider(index, generation);
    if (!c) return false;
    const bool same = c->body == bodyIndex && c->bodyGeneration == bodyGeneration && c->shape == shape &&
                      std::memcmp(c->dims, dims, sizeof(c->dims)) == 0 &&
                      std::memcmp(c->lpos, lpos, sizeof(c->lpos)) == 0 &&
                      std::memcmp(c->lrot, lrot, sizeof(c->lrot)) == 0;
    if (same) return true;
    // changed geometry wakes the old and the new body (prepareSleeping's
    // collider comparison, physics_world.cpp:455-465)
    if (HostBody *b = body(c->body, c->bodyGeneration)) b->wakeUp();
    if (HostBody *b = body(bodyIndex, bodyGeneration)) b->wakeUp();
    c->body = bodyIndex;
    c->bodyGeneration = bodyGeneration;
    c->shape = shape;
    std::memcpy(c->dims, dims, sizeof(c->dims));
    std::memcpy(c->lpos, lpos, sizeof(c->lpos));
    std::memcpy(c->lrot, lrot, sizeof(c->lrot));
    hostDirty_ = true;
    return true;
}

HostBody *World::body(uint32_t index, uint32_t generation) {
    if (index >= bodies.size()) return nullptr;
    HostBody &b = bodies[index];
    if (!b.alive || b.generation != generation) return nullptr;
    return &b;
}

HostCollider *World::collider(uint32_t index, uint32_t generation) {
    if (index >= colliders.size()) return nullptr;
    HostCollider &c = colliders[index];
    if (!c.alive || c.generation != generation) return nullptr;
    return &c;
}

void World::wakeContacts(uint32_t index, uint32_t generation) {
    if (!sleepingEnabled || !lastManifolds_) return;
    const uint32_t M = lastManifolds_;
    std::vector<uint32_t> ba(M), ga(M), bbv(M), gb(M);
    PE_CHECK(cudaMemcpy(ba.data(), mBodyA_.ptr, M * 4, cudaMemcpyDeviceToHost));
    PE_CHECK(cudaMemcpy(ga.data(), mGenA_.ptr, M * 4, cudaMemcpyDeviceToHost));
    PE_CHECK(cudaMemcpy(bbv.data(), mBodyB_.ptr, M * 4, cudaMemcpyDeviceToHost));
    PE_CHECK(cudaMemcpy(gb.data(), mGenB_.ptr, M * 4, cudaMemcpyDeviceToHost));
    for (uint32_t m = 0; m < M; ++m) {
        if (ba[m] == index && ga[m] == generation)
            if (HostBody *o = body(bbv[m], gb[m]); o && !o->isStatic) o->wakeUp();
        if (bbv[m] == index && gb[m] == generation)
            if (HostBody *o = body(ba[m], ga[m]); o && !o->isStatic) o->wakeUp();
    }
}

void World::setSleepingEnabled(bool enabled) {
    if (sleepingEnabled == enabled) return;
    pull();
    sleepingEnabled = enabled;
    // the sleep states start over (quiet times zero, no snapshot) and every
    // live body wakes
    for (HostBody &b : bodies) {
        b.quiet = 0.0f;
        b.snapValid = false;
        if (b.alive) b.wakeUp();
    }
    hostDirty_ = true;
    dropGraphs();
}

std::unique_ptr<World> World::clone() {
    PE_CHECK(cudaSetDevice(device_));
    if (hostDirty_) {
        pull();
        push();
    }
    pull();
    PE_CHECK(cudaStreamSynchronize(stream_));
    auto c = std::make_unique<World>(device_);
    c->gravity[0] = gravity[0];
    c->gravity[1] = gravity[1];
    c->gravity[2] = gravity[2];
    c->algorithm = algorithm;
    c->cellSize = cellSize;
    c->iterations = iterations;
    c->orderMode = orderMode;
    c->sleepingEnabled = sleepingEnabled;
    c->bodies = bodies;
    c->freeBodies = freeBodies;
    c->colliders = colliders;
    c->freeColliders = freeColliders;
    c->hullVerts = hullVerts;
    c->hullOffsets = hullOffsets;
    std::memcpy(c->sleepGravity_, sleepGravity_, sizeof(sleepGravity_));
    c->pairCap_ = pairCap_;
    c->entryCap_ = entryCap_;
    c->mcap_ = mcap_;
    c->cacheNeed_ = std::max(cacheNeed_, cacheCap_);
    c->gridKeyBits_ = gridKeyBits_;
    c->hashGrid_ = hashGrid_;
    c->bodyPairs_ = bodyPairs_;
    c->lastMEstimate_ = lastMEstimate_;
    c->lastRawEstimate_ = lastRawEstimate_;
    c->lastPairs_ = lastPairs_;
    c->lastManifolds_ = lastManifolds_;
    c->counters_ = counters_;
    c->solveSkipped_ = solveSkipped_;
    c->steps_ = steps_;
    c->lastErr_ = lastErr_;
    c->graphsDisabled_ = graphsDisabled_;
    c->push();  // allocates with the same capacities and uploads the bodies
    c->forces_ = forces_;
    c->wakeCheck_ = wakeCheck_;
    cudaStream_t s = stream_;
    auto d2d = [&](void *dst, const void *src, size_t bytes) {
        if (bytes) PE_CHECK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, s));
    };
    const size_t nb = nb_;
    d2d(c->force_.ptr, force_.ptr, nb * sizeof(float4));
    // contacts of the last step, its candidate pairs and solve colours
    const size_t M = lastManifolds_, P = lastPairs_;
    d2d(c->mBodyA_.ptr, mBodyA_.ptr, M * 4);
    d2d(c->mGenA_.ptr, mGenA_.ptr, M * 4);
    d2d(c->mBodyB_.ptr, mBodyB_.ptr, M * 4);
    d2d(c->mGenB_.ptr, mGenB_.ptr, M * 4);
    d2d(c->mCount_.ptr, mCount_.ptr, M * 4);
    d2d(c->mRest_.ptr, mRest_.ptr, M * 4);
    d2d(c->mNormal_.ptr, mNormal_.ptr, M * sizeof(float4));
    d2d(c->mAnchorA_.ptr, mAnchorA_.ptr, 4 * M * sizeof(float4));
    d2d(c->mAnchorB_.ptr, mAnchorB_.ptr, 4 * M * sizeof(float4));
    d2d(c->mImpulse_.ptr, mImpulse_.ptr, 4 * M * sizeof(float4));
    d2d(c->mFeature_.ptr, mFeature_.ptr, 4 * M * 4);
    d2d(c->sColor_.ptr, sColor_.ptr, M * 4);
    d2d(c->pairA_.ptr, pairA_.ptr, P * 4);
    d2d(c->pairB_.ptr, pairB_.ptr, P * 4);
    // warm-start cache (the copy's current cache is its slot cache_)
    uint32_t K = 0;
    PE_CHECK(cudaMemcpyAsync(&K, &cCount_.ptr[cache_], 4, cudaMemcpyDeviceToHost, s));
    PE_CHECK(cudaStreamSynchronize(s));
    K = std::min(K, cacheCap_);
    const int to = c->cache_;
    d2d(c->cKey_[to].ptr, cKey_[cache_].ptr, (size_t)K * 8);
    d2d(c->cGens_[to].ptr, cGens_[cache_].ptr, (size_t)K * 8);
    d2d(c->cA_[to].ptr, cA_[cache_].ptr, (size_t)K * sizeof(float4));
    d2d(c->cB_[to].ptr, cB_[cache_].ptr, (size_t)K * sizeof(float4));
    d2d(c->cT2_[to].ptr, cT2_[cache_].ptr, (size_t)K * 4);
    PE_CHECK(cudaStreamSynchronize(s));
    PE_CHECK(cudaMemcpy(&c->cCount_.ptr[to], &K, 4, cudaMemcpyHostToDevice));
    return c;
}

int World::addHull(const float *verts, uint32_t count) {
    hostDirty_ = true;
    hullVerts.insert(hullVerts.end(), verts, verts + 3 * (size_t)count);
    hullOffsets.push_back((uint32_t)(hullVerts.size() / 3));
    return (int)hullOffsets.size() - 2;
}

// ---------------------------------------------------------- host/device ----
void World::pull() {
    if (!deviceNewer_) return;
    PE_CHECK(cudaSetDevice(device_));
    std::vector<float4> p(nb_), q(nb_), l(nb_), a(nb_);
    std::vector<uint32_t> sf;
    std::vector<float> qt;
    if (nb_) {
        PE_CHECK(cudaMemcpyAsync(p.data(), pos_[cur_].ptr, nb_ * sizeof(float4), cudaMemcpyDeviceToHost, stream_));
        PE_CHECK(cudaMemcpyAsync(q.data(), rot_[cur_].ptr, nb_ * sizeof(float4), cudaMemcpyDeviceToHost, stream_));
        PE_CHECK(cudaMemcpyAsync(l.data(), lin_[cur_].ptr, nb_ * sizeof(float4), cudaMemcpyDeviceToHost, stream_));
        PE_CHECK(cudaMemcpyAsync(a.data(), ang_[cur_].ptr, nb_ * sizeof(float4), cudaMemcpyDeviceToHost, stream_));
        if (sleepingEnabled && sleep_[cur_].ptr) {
            sf.resize(nb_);
            qt.resize(nb_);
            PE_CHECK(cudaMemcpyAsync(sf.data(), sleep_[cur_].ptr, nb_ * 4, cudaMemcpyDeviceToHost, stream_));
            PE_CHECK(cudaMemcpyAsync(qt.data(), quiet_[cur_].ptr, nb_ * 4, cudaMemcpyDeviceToHost, stream_));
        }
        PE_CHECK(cudaStreamSynchronize(stream_));
    }
    for (uint32_t i = 0; i < nb_ && i < bodies.size(); ++i) {
        HostBody &b = bodies[i];
        b.pos[0] = p[i].x; b.pos[1] = p[i].y; b.pos[2] = p[i].z;
        b.rot[0] = q[i].x; b.rot[1] = q[i].y; b.rot[2] = q[i].z; b.rot[3] = q[i].w;
        b.lin[0] = l[i].x; b.lin[1] = l[i].y; b.lin[2] = l[i].z;
        b.ang[0] = a[i].x; b.ang[1] = a[i].y; b.ang[2] = a[i].z;
        // PhysicsWorld::step clears forces of live bodies (physics_world.cpp:766)
        if (b.alive) b.force[0] = b.force[1] = b.force[2] = 0.0f;
        if (!sf.empty()) {
            b.sleeping = (sf[i] & kSleepAsleep) != 0;
            b.wakeRequested = (sf[i] & kSleepWake) != 0;
            b.quiet = qt[i];
        }
        // the end-of-step state edits are compared against (finishSleeping, :506-511)
        b.snapValid = true;
        std::memcpy(b.snapPos, b.pos, sizeof(b.pos));
        std::memcpy(b.snapRot, b.rot, sizeof(b.rot));
        b.snapMass = b.mass;
        b.snapRestitution = b.restitution;
        b.snapFriction = b.friction;
        b.snapStatic = b.isStatic;
    }
    deviceNewer_ = false;
}

void World::computePossiblePairs() {
    // physics_world.cpp:568-581
    std::vector<uint64_t> perBody(bodies.size(), 0);
    uint64_t total = 0, count = 0;
    for (const HostCollider &c : colliders) {
        if (!c.alive || c.body >= bodies.size() || !bodies[c.body].alive || bodies[c.body].generation != c.bodyGeneration)
            continue;
        total += count - perBody[c.body];
        ++perBody[c.body];
        ++count;
    }
    possiblePairs_ = total;
    dynamicAlive_ = 0;
    for (const HostBody &b : bodies)
        if (b.alive && !b.isStatic) ++dynamicAlive_;
}

void World::push() {
    PE_CHECK(cudaSetDevice(device_));
    nb_ = (uint32_t)bodies.size();
    nc_ = (uint32_t)colliders.size();
    ensureCapacity();
    std::vector<float4> p(nb_), q(nb_), l(nb_), a(nb_), f(nb_), mat(nb_), ii(nb_);
    std::vector<uint32_t> flags(nb_), gen(nb_), sf(sleepingEnabled ? nb_ : 0);
    std::vector<float> qt(sleepingEnabled ? nb_ : 0);
    forces_ = false;
    // prepareSleeping (physics_world.cpp:434-452): a gravity change, or an
    // edit of a body's pose, mass, material or static flag since the last
    // step, wakes the body.
    const bool gravityChanged = gravity[0] != sleepGravity_[0] || gravity[1] != sleepGravity_[1] ||
                                gravity[2] != sleepGravity_[2];
    for (uint32_t i = 0; i < nb_; ++i) {
        HostBody &b = bodies[i];
        if (sleepingEnabled) {
            if (b.alive &&
                (gravityChanged || !b.snapValid || b.snapMass != b.mass || b.snapStatic != b.isStatic ||
                 b.snapFriction != b.friction || b.snapRestitution != b.restitution || b.snapPos[0] != b.pos[0] ||
                 b.snapPos[1] != b.pos[1] || b.snapPos[2] != b.pos[2] || b.snapRot[0] != b.rot[0] ||
                 b.snapRot[1] != b.rot[1] || b.snapRot[2] != b.rot[2] || b.snapRot[3] != b.rot[3]))
                b.wakeUp();
            sf[i] = (b.sleeping ? kSleepAsleep : 0u) | (b.wakeRequested ? kSleepWake : 0u);
            qt[i] = b.quiet;
        }
        p[i] = make_float4(b.pos[0], b.pos[1], b.pos[2], 0.0f);
        q[i] = make_float4(b.rot[0], b.rot[1], b.rot[2], b.rot[3]);
        l[i] = make_float4(b.lin[0], b.lin[1], b.lin[2], 0.0f);
        a[i] = make_float4(b.ang[0], b.ang[1], b.ang[2], 0.0f);
        f[i] = make_float4(b.force[0], b.force[1], b.force[2], 0.0f);
        if (b.alive && (b.force[0] != 0.0f || b.force[1] != 0.0f || b.force[2] != 0.0f)) forces_ = true;
        // RigidBody::getInverseMass (rigid_body.hpp:72-75)
        float invMass = b.isStatic || b.mass <= 0.0f ? 0.0f : 1.0f / b.mass;
        mat[i] = make_float4(invMass, b.restitution, b.friction, b.mass);
        ii[i] = make_float4(b.iinv[0], b.iinv[1], b.iinv[2], 0.0f);
        flags[i] = (b.alive ? kBodyAlive : 0u) | (b.isStatic ? kBodyStatic : 0u);
        gen[i] = b.generation;
    }
    upload(pos_[cur_], p, stream_);
    upload(rot_[cur_], q, stream_);
    upload(lin_[cur_], l, stream_);
    upload(ang_[cur_], a, stream_);
    upload(force_, f, stream_);
    upload(mat_, mat, stream_);
    upload(iinv_, ii, stream_);
    upload(bflags_, flags, stream_);
    upload(bgen_, gen, stream_);
    if (sleepingEnabled) {
        upload(sleep_[cur_], sf, stream_);
        upload(quiet_[cur_], qt, stream_);
        wakeCheck_ = true;
    }

    std::vector<uint32_t> cb(nc_), cg(nc_), cf(nc_);
    std::vector<float4> cs(nc_), lp(nc_), lr(nc_);
    dense_ = true;
    localIdentity_ = true;
    bool identity = true;
    for (uint32_t i = 0; i < nc_; ++i) {
        const HostCollider &c = colliders[i];
        cb[i] = c.body;
        cg[i] = c.bodyGeneration;
        cf[i] = (c.alive ? kColliderAlive : 0u) | (c.shape << 8);
        float hw;
        uint32_t hb = c.hull;
        std::memcpy(&hw, &hb, 4);
        cs[i] = make_float4(c.dims[0], c.dims[1], c.dims[2], hw);
        lp[i] = make_float4(c.lpos[0], c.lpos[1], c.lpos[2], 0.0f);
        lr[i] = make_float4(c.lrot[0], c.lrot[1], c.lrot[2], c.lrot[3]);
        if (c.lpos[0] != 0.0f || c.lpos[1] != 0.0f || c.lpos[2] != 0.0f || c.lrot[0] != 0.0f || c.lrot[1] != 0.0f ||
            c.lrot[2] != 0.0f || c.lrot[3] != 1.0f)
            localIdentity_ = false;
        bool valid = c.alive && c.body < nb_ && bodies[c.body].alive && bodies[c.body].generation == c.bodyGeneration;
        if (!valid) dense_ = false;
        if (!valid || c.body != i) identity = false;
    }
    identityColliders_ = identity && nc_ == nb_;
    upload(cbody_, cb, stream_);
    upload(cbgen_, cg, stream_);
    upload(cflags_, cf, stream_);
    upload(cshape_, cs, stream_);
    upload(clpos_, lp, stream_);
    upload(clrot_, lr, stream_);
    std::vector<uint32_t> ho(hullOffsets.begin(), hullOffsets.end());
    std::vector<float4> hv(hullVerts.size() / 3);
    for (size_t k = 0; k < hv.size(); ++k)
        hv[k] = make_float4(hullVerts[3 * k], hullVerts[3 * k + 1], hullVerts[3 * k + 2], 0.0f);
    upload(hullOffset_, ho, stream_);
    upload(hullVerts_, hv, stream_);
    computePossiblePairs();
    PE_CHECK(cudaStreamSynchronize(stream_));
    hostDirty_ = false;
}

void World::ensureScratch(uint32_t maxN) {
    if (maxN <= scratchN_ && wsScan_.ptr) return;
    scratchN_ = maxN;
    // Look-back state per tile; the smallest tiles (the narrowphase's) hold
    // kMinLookbackTile items.  The pair kernel's states (256-body tiles) may
    // sit in front of the narrowphase's so that both are cleared ahead.
    wsScan_.reserve((maxN + kMinLookbackTile - 1) / kMinLookbackTile + (maxN + 255) / 256 + 32);
    wsSortHist_.reserve(256 * 8 + 64);
    wsSortState_.reserve(scratchBytesSort(maxN) / sizeof(uint32_t) + 16);
    ws_.scanState = wsScan_.ptr;
    ws_.sortHist = wsSortHist_.ptr;
    ws_.sortState = wsSortState_.ptr;
}

void World::ensureCapacity() {
    dropGraphs();
    const uint32_t nb = std::max<uint32_t>(nb_, 1), nc = std::max<uint32_t>(nc_, 1);
    for (int k = 0; k < 2; ++k) {
        pos_[k].reserve(nb);
        rot_[k].reserve(nb);
        lin_[k].reserve(nb);
        ang_[k].reserve(nb);
    }
    if (sleepingEnabled) {
        for (int k = 0; k < 2; ++k) {
            sleep_[k].reserve(nb);
            quiet_[k].reserve(nb);
        }
        sParent_.reserve(nb);
        sIsland_.reserve(nb);
        sQuietMin_.reserve(nb);
        sleepErr_.reserve(1);
    }
    aabbMin_.reserve(nc);
    aabbMax_.reserve(nc);
    npRec_.reserve(4 * (size_t)nc);
    collectFlags_.reserve(nc);
    collectPos_.reserve(nc);
    inSlot_.reserve(nc);
    inMin_.reserve(nc);
    inMax_.reserve(nc);
    sapKeys_.reserve(nc);
    sapVals_.reserve(nc);
    sapKeyOf_.reserve(nc);
    sapWords_.reserve(2);
    bbKeyTmp32_.reserve(nc);
    bbValTmp_.reserve(nc);
    bbMinX_.reserve(nc);
    bbMaxX_.reserve(nc);
    bbYZ_.reserve(nc);
    bbIdx_.reserve(nc);
    bbLen_.reserve(nc);
    bbOff_.reserve(nc);
    bbWidth_.reserve(nc);
    bbWidthTmp_.reserve(nc);
    bbFirst_.reserve(nc);
    bbCellCount_.reserve(nc);
    bbInGrid_.reserve(nc);
    bbOverflow_.reserve(nc);
    bbEntryOff_.reserve(nc);
    bbCounters_.reserve(4);
    if (entryCap_ < 8u * nc) entryCap_ = std::max<uint32_t>(65536, 8u * nc);
    bbEntryKeys_.reserve(entryCap_);
    bbEntryKeysTmp_.reserve(entryCap_);
    bbEntryVals_.reserve(entryCap_);
    bbEntryValsTmp_.reserve(entryCap_);
    // hashed grid buckets: a power of two, about two per collider
    uint32_t logB = 10;
    while ((1u << logB) < 2u * nc && logB < 30) ++logB;
    bbBucketHead_.reserve(1u << logB);
    bbEntryNext_.reserve(entryCap_);
    bbEntryRec_.reserve(entryCap_);
    bbCand_.reserve(2 * (size_t)nc);
    bb_ = BroadBuffers{bbKeyTmp32_.ptr, bbValTmp_.ptr, bbMinX_.ptr, bbMaxX_.ptr, bbYZ_.ptr, bbIdx_.ptr, bbLen_.ptr,
                       bbOff_.ptr, bbWidth_.ptr, bbWidthTmp_.ptr, bbFirst_.ptr, bbCellCount_.ptr, bbInGrid_.ptr,
                       bbOverflow_.ptr, bbEntryOff_.ptr, bbEntryKeys_.ptr, bbEntryKeysTmp_.ptr, bbEntryVals_.ptr,
                       bbEntryValsTmp_.ptr, entryCap_, gridKeyBits_, bbCounters_.ptr, bbBucketHead_.ptr,
                       bbEntryNext_.ptr, false, nullptr, 0, logB, false, bbEntryRec_.ptr, bbCand_.ptr};

    if (pairCap_ < 4u * nc) pairCap_ = std::max<uint32_t>(65536, 4u * nc);
    pairKeys_.reserve(pairCap_);
    pairKeysTmp_.reserve(pairCap_);
    pairFlags_.reserve(pairCap_);
    pairPos_.reserve(pairCap_);
    pairA_.reserve(pairCap_);
    pairB_.reserve(pairCap_);
    pairCounters_.reserve(4);
    pb_ = PairBuffers{pairKeys_.ptr, pairKeysTmp_.ptr, pairCap_, 32u, false, false, pairFlags_.ptr, pairPos_.ptr,
                      pairA_.ptr, pairB_.ptr, pairCounters_.ptr};

    if (mcap_ < pairCap_) mcap_ = pairCap_;
    const uint32_t m = mcap_;
    // The last step's manifolds survive growth (contacts(), and the wake pass
    // before the next step reads them).
    const size_t keep = lastManifolds_;
    reserveKeep(mBodyA_, m, keep);
    reserveKeep(mGenA_, m, keep);
    reserveKeep(mBodyB_, m, keep);
    reserveKeep(mGenB_, m, keep);
    reserveKeep(mCount_, m, keep);
    reserveKeep(mRest_, m, keep);
    reserveKeep(mNormal_, m, keep);
    reserveKeep(mAnchorA_, 4 * (size_t)m, 4 * keep);
    reserveKeep(mAnchorB_, 4 * (size_t)m, 4 * keep);
    reserveKeep(mImpulse_, 4 * (size_t)m, 4 * keep);
    reserveKeep(mFeature_, 4 * (size_t)m, 4 * keep);

    sBest_.reserve(nb);
    sUsed_.reserve(2 * (size_t)nb);
    sColor_.reserve(m);
    sDyn_.reserve(m);
    sColorCount_.reserve(kMaxColors);
    sColorStart_.reserve(m);
    sOrderKeys_.reserve(m);
    sOrderKeysTmp_.reserve(m);
    sOrder_.reserve(m);
    sOrderTmp_.reserve(m);
    sPm_.reserve(m);
    sPmI_.reserve(6 * (size_t)m);
    sPp_.reserve((size_t)kPreparedVec4 * 4 * m);
    sPimp_.reserve(4 * (size_t)m);
    sPn_.reserve(m);
    sPbody_.reserve(m);
    sPcount_.reserve(m);
    sCacheKeys_.reserve(m);
    sCacheKeysTmp_.reserve(m);
    sCacheVals_.reserve(m);
    sCacheValsTmp_.reserve(m);
    sCacheCounts_.reserve(m);
    sCacheOff_.reserve(m);
    sBar_.reserve(2);
    sCounters_.reserve(4);
    sStageSlot_.reserve(m);
    sStageBody_.reserve(2 * (size_t)m + 64);
    sIslandList_.reserve((size_t)kIslandMax * nb);
    sIslPar_.reserve(2 * (size_t)nb);
    sIslOff_.reserve(nb);
    sIslRoot_.reserve(m);
    sIslSlot_.reserve(m);
    sIslList_.reserve(m);
    sIslRoots_.reserve(m);
    sIslLone_.reserve(m);
    sIslCounters_.reserve(kIslCounterWords);
    sIslKeys_.reserve(m);
    sIslKeysTmp_.reserve(m);
    sIslSort_.reserve(2 * (size_t)m);
    sIslLink_.reserve(nb);
    sIslSize_.reserve(nb);
    sIslandRec_.reserve((size_t)kIslandMax * nb);
    sPathHint_.reserve(1);
    sb_ = SolverBuffers{m,
                        sBest_.ptr,
                        sUsed_.ptr,
                        sEpoch_.ptr,
                        sColor_.ptr,
                        sDyn_.ptr,
                        sColorCount_.ptr,
                        sColorStart_.ptr,
                        sOrderKeys_.ptr,
                        sOrderKeysTmp_.ptr,
                        sOrder_.ptr,
                        sOrderTmp_.ptr,
                        sPm_.ptr,
                        sPmI_.ptr,
                        sPp_.ptr,
                        sPimp_.ptr,
                        sPn_.ptr,
                        sPbody_.ptr,
                        sPcount_.ptr,
                        sCacheKeys_.ptr,
                        sCacheKeysTmp_.ptr,
                        sCacheVals_.ptr,
                        sCacheValsTmp_.ptr,
                        sCacheCounts_.ptr,
                        sCacheOff_.ptr,
                        sBar_.ptr,
                        sCounters_.ptr,
                        sStageSlot_.ptr,
                        sStageBody_.ptr,
                        sIslandList_.ptr,
                        sIslPar_.ptr,
                        sIslOff_.ptr,
                        sIslRoot_.ptr,
                        sIslSlot_.ptr,
                        sIslList_.ptr,
                        sIslRoots_.ptr,
                        sIslLone_.ptr,
                        sIslKeys_.ptr,
                        sIslKeysTmp_.ptr,
                        sIslSort_.ptr,
                        sIslCounters_.ptr,
                        sIslLink_.ptr,
                        sIslSize_.ptr,
                        sIslandRec_.ptr,
                        sPathHint_.ptr};

    // Warm-start caches keep their contents when they grow.
    const uint32_t needCache = std::max(4 * m, cacheNeed_);
    if (cacheCap_ < needCache) {
        for (int k = 0; k < 2; ++k) {
            DeviceArray<unsigned long long> nk, ng;
            DeviceArray<float4> na, nbb;
            DeviceArray<float> nt;
            nk.reserve(needCache);
            ng.reserve(needCache);
            na.reserve(needCache);
            nbb.reserve(needCache);
            nt.reserve(needCache);
            if (cacheCap_) {
                PE_CHECK(cudaMemcpy(nk.ptr, cKey_[k].ptr, cacheCap_ * sizeof(unsigned long long), cudaMemcpyDeviceToDevice));
                PE_CHECK(cudaMemcpy(ng.ptr, cGens_[k].ptr, cacheCap_ * sizeof(unsigned long long), cudaMemcpyDeviceToDevice));
                PE_CHECK(cudaMemcpy(na.ptr, cA_[k].ptr, cacheCap_ * sizeof(float4), cudaMemcpyDeviceToDevice));
                PE_CHECK(cudaMemcpy(nbb.ptr, cB_[k].ptr, cacheCap_ * sizeof(float4), cudaMemcpyDeviceToDevice));
                PE_CHECK(cudaMemcpy(nt.ptr, cT2_[k].ptr, cacheCap_ * sizeof(float), cudaMemcpyDeviceToDevice));
            }
            std::swap(cKey_[k].ptr, nk.ptr);
            std::swap(cKey_[k].count, nk.count);
            std::swap(cGens_[k].ptr, ng.ptr);
            std::swap(cGens_[k].count, ng.count);
            std::swap(cA_[k].ptr, na.ptr);
            std::swap(cA_[k].count, na.count);
            std::swap(cB_[k].ptr, nbb.ptr);
            std::swap(cB_[k].count, nbb.count);
            std::swap(cT2_[k].ptr, nt.ptr);
            std::swap(cT2_[k].count, nt.count);
        }
        cacheCap_ = needCache;
    }
    if (sleepingEnabled) {
        // the solver's entries before the merge with the carried ones
        tKey_.reserve(cacheCap_);
        tGens_.reserve(cacheCap_);
        tA_.reserve(cacheCap_);
        tB_.reserve(cacheCap_);
        tT2_.reserve(cacheCap_);
        tCount_.reserve(1);
        carry_.reserve(cacheCap_);
        carryPos_.reserve(cacheCap_);
        carryTotal_.reserve(1);
    }
    ensureScratch(std::max({nc, nb, pairCap_, entryCap_, m, cacheCap_}));
}

void World::ensureLbvh() {
    const uint32_t n = std::max<uint32_t>(nc_, 2);
    lbKeys_.reserve(n);
    lbKeysTmp_.reserve(n);
    lbChildL_.reserve(n);
    lbChildR_.reserve(n);
    lbParent_.reserve(n);
    lbLeafParent_.reserve(n);
    lbRangeMax_.reserve(n);
    lbVisit_.reserve(n);
    lbBox_.reserve(8);
    lbLeafMn_.reserve(n);
    lbLeafMx_.reserve(n);
    lbNodeMn_.reserve(n);
    lbNodeMx_.reserve(n);
    lb_ = LbvhBuffers{lbKeys_.ptr,     lbKeysTmp_.ptr, lbChildL_.ptr,  lbChildR_.ptr,   lbParent_.ptr,
                      lbLeafParent_.ptr, lbRangeMax_.ptr, lbVisit_.ptr,  lbLeafMn_.ptr,   lbLeafMx_.ptr,
                      lbNodeMn_.ptr,   lbNodeMx_.ptr,  lbBox_.ptr};
}

WorldView World::view(float dt) {
    WorldView w{};
    w.nb = nb_;
    w.nc = nc_;
    w.cur = BodyState{pos_[cur_].ptr, rot_[cur_].ptr, lin_[cur_].ptr, ang_[cur_].ptr};
    w.nxt = BodyState{pos_[1 - cur_].ptr, rot_[1 - cur_].ptr, lin_[1 - cur_].ptr, ang_[1 - cur_].ptr};
    w.force = forces_ ? force_.ptr : nullptr;
    w.force3 = rawForces_ ? xfer3_.ptr : nullptr;
    w.force3n = rawForces_ ? force3n_ : 0u;
    w.pos3 = packPoses_ ? posOut_.ptr : nullptr;
    w.io = ioMode_ ? ioDev_ : nullptr;
    w.mat = mat_.ptr;
    w.iinv = iinv_.ptr;
    w.bflags = bflags_.ptr;
    w.bgen = bgen_.ptr;
    w.cbody = cbody_.ptr;
    w.cbgen = cbgen_.ptr;
    w.cflags = cflags_.ptr;
    w.cshape = cshape_.ptr;
    w.clpos = localIdentity_ ? nullptr : clpos_.ptr;
    w.clrot = localIdentity_ ? nullptr : clrot_.ptr;
    w.hullOffset = hullOffset_.ptr;
    w.hullVerts = hullVerts_.ptr;
    w.aabbMin = aabbMin_.ptr;
    w.aabbMax = aabbMax_.ptr;
    w.npRec = npRec_.ptr;
    w.gx = gravity[0];
    w.gy = gravity[1];
    w.gz = gravity[2];
    w.dt = dt;
    if (sleepingEnabled) {
        w.sleepMode = 1;
        w.sleepIn = sleep_[cur_].ptr;
        w.sleepOut = sleep_[1 - cur_].ptr;
        w.quietIn = quiet_[cur_].ptr;
        w.quietOut = quiet_[1 - cur_].ptr;
        w.sleepParent = sParent_.ptr;
        w.sleepIsland = sIsland_.ptr;
        w.sleepQuietMin = sQuietMin_.ptr;
    }
    return w;
}

ManifoldView World::manifoldView() {
    return ManifoldView{mBodyA_.ptr, mGenA_.ptr,     mBodyB_.ptr,   mGenB_.ptr,    mNormal_.ptr, mRest_.ptr,
                        mCount_.ptr, mAnchorA_.ptr, mAnchorB_.ptr, mImpulse_.ptr, mFeature_.ptr};
}

CacheView World::cacheView(int which) {
    return CacheView{cKey_[which].ptr, cGens_[which].ptr, cA_[which].ptr, cB_[which].ptr, cT2_[which].ptr};
}

void World::runPipeline(float dt) {
    cudaStream_t s = stream_;
    WorldView w = view(dt);
    DevStats *st = stats_.ptr;
    const bool sap = algorithm == 0;
    // Dense hashed grid with per-body pairs: the integrate kernel clears the
    // bucket heads and the insert kernel the look-back states of the pair and
    // narrowphase kernels (three memset nodes fewer per step).
    const bool fused = dense_ && !sap && bb_.hashed && pb_.bodyPath;
    const uint32_t pairTiles = (nc_ + 255) / 256 + 1;
    const uint32_t narrowOff = pairTiles + 1, narrowTiles = (pb_.cap + kMinLookbackTile - 1) / kMinLookbackTile + 1;
    bb_.headsCleared = fused;
    bb_.zeroState = fused ? ws_.scanState : nullptr;
    bb_.nZeroState = fused ? narrowOff + narrowTiles + 1 : 0;
    // dense SAP keeps last step's order and skips the sort while it still holds
    const SapCoherence coh{sapKeyOf_.ptr, sapWords_.ptr, sapWords_.ptr + 1};
    if (dense_) {
        launchIntegrateAabb(w, sap ? sapKeyOf_.ptr : nullptr, nullptr, st, nc_, s, fused ? bb_.bucketHead : nullptr,
                            fused ? (1u << bb_.logBuckets) : 0u);
    } else {
        launchIntegrateAabb(w, nullptr, nullptr, st, 0u, s);
        launchCollect(w, collectFlags_.ptr, collectPos_.ptr, inMin_.ptr, inMax_.ptr, inSlot_.ptr,
                      sap ? sapKeys_.ptr : nullptr, sapVals_.ptr, &st->inputCount, ws_, &st->err, s);
    }
    BroadInput in{dense_ ? aabbMin_.ptr : inMin_.ptr, dense_ ? aabbMax_.ptr : inMax_.ptr, &st->inputCount, nc_};
    const PairMapping mapping{dense_ ? nullptr : inSlot_.ptr, cbody_.ptr, cbgen_.ptr};
    bool finalized = false;
    if (sap) finalized = launchSap(in, sapKeys_.ptr, sapVals_.ptr, bb_, pb_, st, ws_, s, dense_ ? &coh : nullptr,
                                   &mapping);
    else if (algorithm == 2) launchLbvh(in, lb_, pb_, st, ws_, s);
    else launchGrid(in, cellSize, bb_, pb_, st, ws_, s);
    if (!sap && pb_.bodyPath)
        launchGridBodyPairs(in, bb_, pb_, mapping.inSlot, cbody_.ptr, cbgen_.ptr, st, ws_, s, fused);
    else if (!finalized)
        launchPairsFinalize(mapping.inSlot, cbody_.ptr, cbgen_.ptr, pb_, st, ws_, s);
    ManifoldView mv = manifoldView();
    launchNarrowphase(w, pb_, mv, mcap_, st, ws_, s, fused ? ws_.scanState + narrowOff : nullptr, fused);
    const bool sleeping = sleepingEnabled;
    // contacts can wake islands after the gravity pass (physics_world.cpp:741-748)
    if (sleeping) launchSleepContacts(w, mv, st, mcap_, bflags_.ptr, s);
    // with sleeping on the solver's cache entries are merged with the carried
    // entries of sleeping contacts into the next cache
    const CacheView tmp{tKey_.ptr, tGens_.ptr, tA_.ptr, tB_.ptr, tT2_.ptr};
    launchSolver(w, mv, cacheView(cache_), &cCount_.ptr[cache_], sleeping ? tmp : cacheView(1 - cache_),
                 sleeping ? tCount_.ptr : &cCount_.ptr[1 - cache_], cacheCap_, sb_, iterations, orderMode, coopBlocks_,
                 blockSolver_, blockM_, identityColliders_, st, ws_, s);
    if (sleeping)
        launchCacheCarry(w, cacheView(cache_), &cCount_.ptr[cache_], tmp, tCount_.ptr, cacheView(1 - cache_),
                         &cCount_.ptr[1 - cache_], cacheCap_, carry_.ptr, carryPos_.ptr, carryTotal_.ptr, st, ws_, s);
    // the last kernel's last block copies the counters to the pinned host
    // mirror (the device writes it directly); with no bodies a copy node does
    if (nb_) {
        launchIntegratePose(w, s, st, sleeping ? nullptr : hostStats_, poseDone_.ptr);
        if (sleeping) launchSleepFinish(w, st, hostStats_, poseDone_.ptr, s);
    } else {
        PE_CHECK(cudaMemcpyAsync(hostStats_, st, sizeof(DevStats), cudaMemcpyDeviceToHost, s));
    }
}

bool World::finishStep() {
    PE_CHECK(cudaStreamSynchronize(stream_));
    const DevStats &h = *hostStats_;
    lastErr_ = h.err;
    if (h.err & (kErrTimeout | kErrColors | kErrEntryCapacity | kErrTreeDepth)) {
        throw std::runtime_error(std::string("step failed on the device: ") +
                                 ((h.err & kErrTimeout) ? "a bounded wait timed out" :
                                  (h.err & kErrColors) ? "the solver colouring exceeded its round limit" :
                                  (h.err & kErrTreeDepth) ? "a bounding-volume tree traversal outgrew its stack" :
                                                            "grid cell range exceeds 64 key bits"));
    }
    bool retry = false, grew = false;
    if (h.err & kErrHashRange) {
        // A cell coordinate beyond the hashed grid's 21-bit range: use the
        // sorted grid from now on.
        hashGrid_ = false;
        retry = true;
    }
    if (h.err & kErrBodyPairs) {
        // A body had more grid partners than the per-body path holds: this
        // world uses the sort-based pair path from now on.
        bodyPairs_ = false;
        retry = true;
    }
    if (h.err & kErrCacheCapacity) {
        // carried sleeping entries and the solver's entries overflowed the cache
        cacheNeed_ = grow(h.carried + 4 * std::max(h.manifolds, 1u), cacheCap_);
        retry = grew = true;
    }
    if (h.err & kErrSmallPath) {
        // A single-block path or the sorted key width was too small: re-run with
        // the sizes this attempt measured.
        lastMEstimate_ = std::max(lastMEstimate_, h.manifolds);
        lastRawEstimate_ = std::max(lastRawEstimate_, h.rawPairs);
        // the cluster solver holds kMaxColors colour ranges: more colours take
        // the multi-kernel path
        if (h.colors > (uint32_t)kMaxColors) wideColors_ = true;
        if (h.cellKeyBits > gridKeyBits_) gridKeyBits_ = std::min<uint32_t>(64, 8 * ((h.cellKeyBits + 9) / 8));
        retry = true;
    }
    if (h.rawPairs > pairCap_) {
        pairCap_ = grow(h.rawPairs, pairCap_);
        retry = grew = true;
    }
    if (h.gridEntryCount > entryCap_) {
        entryCap_ = grow(h.gridEntryCount, entryCap_);
        retry = grew = true;
    }
    if (h.manifolds > mcap_ || h.pairs > mcap_) {
        mcap_ = grow(std::max(h.manifolds, h.pairs), mcap_);
        retry = grew = true;
    }
    if (retry) {
        if (grew) ensureCapacity();
        return false;
    }
    StepCounters &c = counters_;
    c = StepCounters{};
    c.possiblePairs = possiblePairs_;
    c.candidatePairs = h.pairs;
    c.contactCount = h.manifolds;
    c.solvedContactCount = h.solved;
    c.awakeBodyCount = sleepingEnabled ? h.awakeBodies : dynamicAlive_;
    c.sleepingBodyCount = sleepingEnabled ? h.sleepingBodies : 0;
    if (sleepingEnabled) std::memcpy(sleepGravity_, gravity, sizeof(sleepGravity_));
    c.xWindow = h.xWindow;
    c.aabbPairs = h.uniquePairs;
    c.gridComparisons = h.gridComparisons;
    c.gridEntries = algorithm == 1 ? h.gridEntryCount : 0;
    c.gridOverflow = algorithm == 1 ? h.overflowCount : 0;
    c.cellSize = algorithm == 1 ? h.cellSize : 0.0;
    for (int k = 0; k < 4; ++k) {
        c.npCandidates[k] = h.npCandidates[k];
        c.npContacts[k] = h.npContacts[k];
    }
    c.preparedPoints = h.preparedPoints;
    c.warmComparisons = h.warmComparisons;
    c.warmMatches = h.warmMatches;
    c.velocityPointVisits = h.preparedPoints * (uint64_t)iterations;
    // with every body asleep the solver ran on no manifold: every manifold has
    // colour 0 (it has no moving body)
    solveSkipped_ = sleepingEnabled && h.solveCount == 0;
    c.colors = orderMode == 0 ? h.manifolds : solveSkipped_ ? (h.manifolds ? 1u : 0u) : h.colors;
    c.colorRounds = h.colorRounds;
    // gap after the narrowphase, prepare kernel, gap, cluster kernel phases,
    // gap before the pose kernel (zeros when the one-cluster solver did not run)
    {
        const unsigned long long *t = h.solverStamp;
        auto span = [&](unsigned long long t0, unsigned long long t1) {
            return (t[0] && t0 && t1 > t0) ? (t1 - t0) * 1e-6 : 0.0;
        };
        const unsigned long long last = t[7] ? t[7] : t[5];
        c.solverPhaseMs[0] = span(h.stamp[3], t[0]);
        for (int k = 0; k < 5; ++k) c.solverPhaseMs[k + 1] = span(t[k], t[k + 1]);
        c.solverPhaseMs[6] = span(t[5], t[7]);
        c.solverPhaseMs[7] = span(last, h.stamp[4]);
    }
    c.epaFailures = h.epaFailures;
    c.points = h.points;
    lastPairs_ = h.pairs;
    lastManifolds_ = h.manifolds;
    lastMEstimate_ = h.manifolds;
    lastRawEstimate_ = h.rawPairs;
    wideColors_ = orderMode != 0 && !solveSkipped_ && h.colors > (uint32_t)kMaxColors;
    // Cell-key width: whole bytes with at least two bits of slack, widened
    // early so the captured graph rarely changes.
    if (algorithm == 1) {
        uint32_t want = std::min<uint32_t>(64, 8 * ((h.cellKeyBits + 9) / 8));
        if (want > gridKeyBits_ || want + 8 < gridKeyBits_) gridKeyBits_ = want;
    }
    cur_ = 1 - cur_;
    cache_ = 1 - cache_;
    deviceNewer_ = true;
    ++steps_;
    return true;
}

bool World::GraphKey::operator==(const GraphKey &o) const {
    return nb == o.nb && nc == o.nc && pairCap == o.pairCap && entryCap == o.entryCap && mcap == o.mcap &&
           cacheCap == o.cacheCap && dt == o.dt && gx == o.gx && gy == o.gy && gz == o.gz &&
           algorithm == o.algorithm && iterations == o.iterations && orderMode == o.orderMode &&
           coopBlocks == o.coopBlocks && blockSolver == o.blockSolver && blockM == o.blockM && pairBits == o.pairBits &&
           blockPairs == o.blockPairs && bodyPairs == o.bodyPairs && hashed == o.hashed && gridKeyBits == o.gridKeyBits && cellSize == o.cellSize && dense == o.dense &&
           localIdentity == o.localIdentity && forces == o.forces && identityColliders == o.identityColliders &&
           sleeping == o.sleeping && rawForces == o.rawForces && packPoses == o.packPoses && ioMode == o.ioMode &&
           force3n == o.force3n;
}

World::GraphKey World::currentKey(float dt) const {
    GraphKey k{};
    k.nb = nb_;
    k.nc = nc_;
    k.pairCap = pairCap_;
    k.entryCap = entryCap_;
    k.mcap = mcap_;
    k.cacheCap = cacheCap_;
    k.dt = dt;
    k.gx = gravity[0];
    k.gy = gravity[1];
    k.gz = gravity[2];
    k.algorithm = algorithm;
    k.iterations = iterations;
    k.orderMode = orderMode;
    k.coopBlocks = coopBlocks_;
    k.blockSolver = blockSolver_;
    k.blockM = blockM_;
    k.pairBits = pb_.bits;
    k.blockPairs = pb_.blockPath;
    k.bodyPairs = pb_.bodyPath;
    k.hashed = bb_.hashed;
    k.gridKeyBits = bb_.keyBits;
    k.cellSize = cellSize;
    k.dense = dense_;
    k.localIdentity = localIdentity_;
    k.forces = forces_;
    k.identityColliders = identityColliders_;
    k.sleeping = sleepingEnabled;
    k.rawForces = rawForces_;
    k.packPoses = packPoses_;
    k.ioMode = ioMode_;
    k.force3n = rawForces_ ? force3n_ : 0u;
    return k;
}

void World::dropGraphs() {
    for (int p = 0; p < 2; ++p)
        if (graph_[p]) {
            cudaGraphExecDestroy(graph_[p]);
            graph_[p] = nullptr;
        }
}

// Enqueues one step: through a captured graph when possible, else directly.
// Returns the number of engine kernels the step launches.
unsigned long long World::launchStep(float dt) {
    // Cooperative solver grid: every block the device holds at once.  The
    // grid-wide colour sweeps deal each colour's manifolds over all blocks, so
    // a colour of a few thousand manifolds keeps a warp or two busy on every
    // SM rather than filling a few SMs (measured: 0.80 -> 0.58 ms per step on
    // the 10,000-body field, grids sized by manifold count before).
    coopBlocks_ = maxCooperativeBlocks(smCount_);
    // Small manifold counts run the single-block solver (with headroom over
    // the last step's count; an overflow re-runs the step on the full path).
    blockSolver_ = lastMEstimate_ + lastMEstimate_ / 4 + 64 <= kBlockMaxManifolds && nb_ <= kBlockMaxBodies &&
                   !wideColors_;
    blockM_ = 64;
    while (blockM_ < lastMEstimate_ + lastMEstimate_ / 4 + 64 && blockM_ < kBlockMaxManifolds) blockM_ <<= 1;
    // Pair keys need bits for input indices < nc; the small finalize path is
    // used while the last raw pair count leaves headroom.
    uint32_t bits = 1;
    while (bits < 32 && (1ull << bits) < (unsigned long long)std::max<uint32_t>(nc_, 2)) ++bits;
    pb_.bits = bits;
    pb_.blockPath = lastRawEstimate_ + lastRawEstimate_ / 4 + 256 <= kBlockPreferredPairs;
    pb_.bodyPath = algorithm == 1 && bodyPairs_;
    bb_.hashed = pb_.bodyPath && cellSize > 0.0 && hashGrid_;
    bb_.keyBits = gridKeyBits_;
    if (graphsDisabled_) {
        const unsigned long long l0 = g_kernelLaunches;
        runPipeline(dt);
        lastGraphed_ = false;
        return g_kernelLaunches - l0;
    }
    const int p = cur_;
    const GraphKey key = currentKey(dt);
    if (!graph_[p] || !(graphKey_[p] == key)) {
        if (graph_[p]) {
            cudaGraphExecDestroy(graph_[p]);
            graph_[p] = nullptr;
        }
        const unsigned long long l0 = g_kernelLaunches;
        cudaGraph_t g = nullptr;
        PE_CHECK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        try {
            runPipeline(dt);
        } catch (const std::exception &ex) {
            graphError_ = std::string("capture: ") + ex.what();
            cudaStreamEndCapture(stream_, &g);
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            graphsDisabled_ = true;  // capture refused: launch directly from now on
            return launchStep(dt);
        }
        cudaError_t e = cudaStreamEndCapture(stream_, &g);
        if (e != cudaSuccess || !g) {
            graphError_ = std::string("capture: ") + cudaGetErrorString(e);
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            graphsDisabled_ = true;
            return launchStep(dt);
        }
        e = cudaGraphInstantiate(&graph_[p], g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            graphError_ = std::string("instantiate: ") + cudaGetErrorString(e);
            cudaGetLastError();
            graph_[p] = nullptr;
            graphsDisabled_ = true;
            return launchStep(dt);
        }
        graphKey_[p] = key;
        graphLaunches_[p] = g_kernelLaunches - l0;
    }
    PE_CHECK(cudaGraphLaunch(graph_[p], stream_));
    lastGraphed_ = true;
    return graphLaunches_[p];
}

void World::step(float dt) { runStep(dt, nullptr, 0, nullptr, nullptr); }

void World::stepIO(const float *forces, uint32_t n, float dt, float *positions, float *rotations) {
    runStep(dt, forces, n, positions, rotations);
}

void World::runStep(float dt, const float *forces, uint32_t nForces, float *positions, float *rotations) {
    PE_CHECK(cudaSetDevice(device_));
    if (sleepingEnabled && (gravity[0] != sleepGravity_[0] || gravity[1] != sleepGravity_[1] ||
                            gravity[2] != sleepGravity_[2]))
        hostDirty_ = true;  // a gravity change wakes every body (physics_world.cpp:439-451)
    if (hostDirty_) {
        pull();
        push();
    }
    if (algorithm == 2) ensureLbvh();  // before any capture: allocation is not captured
    // Step I/O without extra kernels: the step reads the caller's forces where
    // they land and writes packed positions from its pose kernel.  With
    // sleeping on, forces go through the expanding kernel (it wakes bodies).
    // When every array the caller hands over is addressable by the device
    // (pinned host memory, or device memory of this device), the step reads and
    // writes them in place through the I/O descriptor: no copy operations.
    rawForces_ = packPoses_ = ioMode_ = false;
    force3n_ = 0;
    {
        const bool staged = forces && nForces && (sleepingEnabled || forces_);
        const void *fDev = nullptr;
        void *pDev = nullptr, *rDev = nullptr;
        bool direct = !staged;
        if (direct && forces && nForces) direct = (fDev = deviceAddress(forces, 4)) != nullptr;
        if (direct && positions && nb_) direct = (pDev = deviceAddress(positions, 4)) != nullptr;
        if (direct && rotations && nb_) direct = (rDev = deviceAddress(rotations, 16)) != nullptr;
        if (direct && (fDev || pDev || rDev)) {
            ioHost_->force3 = static_cast<const float *>(fDev);
            ioHost_->force3n = fDev ? std::min<uint32_t>(nForces, nb_) : 0u;
            ioHost_->pos3 = static_cast<float *>(pDev);
            ioHost_->rot4 = static_cast<float4 *>(rDev);
            ioMode_ = true;
            forces = nullptr;  // handled in place
            nForces = 0;
        }
    }
    if (forces && nForces) {
        if (sleepingEnabled || forces_) {  // forces_: forces written earlier for this step
            stageForces(forces, nForces);
        } else {
            force3n_ = std::min<uint32_t>(nForces, nb_);
            xfer3_.reserve(3 * (size_t)std::max<uint32_t>(nb_, 1));
            if (force3n_)
                PE_CHECK(cudaMemcpyAsync(xfer3_.ptr, forces, 3 * (size_t)force3n_ * sizeof(float),
                                         cudaMemcpyHostToDevice, stream_));
            rawForces_ = force3n_ > 0;
        }
    }
    if (positions && nb_ && !ioMode_) {
        posOut_.reserve(3 * (size_t)nb_);
        packPoses_ = true;
    }
    if (sleepingEnabled && wakeCheck_) {
        // prepareSleeping's wake pass over the last step's contacts, on the
        // committed state (outside the step's graph: a re-run of the step
        // must not repeat it)
        WorldView w = view(dt);
        launchSleepWake(w, manifoldView(), lastManifolds_, mcap_, sleep_[cur_].ptr, quiet_[cur_].ptr, sleepErr_.ptr,
                        stream_);
        uint32_t err = 0;
        PE_CHECK(cudaMemcpyAsync(&err, sleepErr_.ptr, 4, cudaMemcpyDeviceToHost, stream_));
        PE_CHECK(cudaStreamSynchronize(stream_));
        if (err) throw std::runtime_error("step failed on the device: a bounded wait timed out");
        wakeCheck_ = false;
    }
    for (int attempt = 0; attempt < 8; ++attempt) {
        const unsigned long long launches = launchStep(dt);
        // poses of this attempt's output copy, read back under the same
        // synchronisation as the step (a re-run attempt copies them again)
        if (nb_ && positions && !ioMode_)
            PE_CHECK(cudaMemcpyAsync(positions, posOut_.ptr, 3 * (size_t)nb_ * sizeof(float), cudaMemcpyDeviceToHost,
                                     stream_));
        if (nb_ && rotations && !ioMode_) enqueuePoses(1 - cur_, nullptr, rotations);
        if (finishStep()) {
            rawForces_ = packPoses_ = ioMode_ = false;
            // device and stage times from the stamps the stage kernels wrote
            // (no event nodes or queries on the step's path; 0 when a stage ran
            // no stamping kernel this step): integrate start to pose end
            float st[5] = {0, 0, 0, 0, 0};
            const unsigned long long *t = hostStats_->stamp;
            for (int k = 0; k < 5; ++k) st[k] = t[k + 1] > t[k] ? (float)((t[k + 1] - t[k]) * 1e-6) : 0.0f;
            counters_.gpuMs = t[0] && t[5] > t[0] ? (t[5] - t[0]) * 1e-6 : 0.0;
            counters_.integrateMs = st[0];
            counters_.broadphaseMs = st[1];
            counters_.narrowphaseMs = st[2];
            counters_.solverMs = st[3];
            counters_.poseMs = st[4];
            counters_.kernelLaunches = launches;
            counters_.graphed = lastGraphed_;
            forces_ = false;  // PhysicsWorld::step clears forces (physics_world.cpp:766)
            return;
        }
    }
    throw std::runtime_error("step buffers kept overflowing");
}

float4 *World::pinnedBuffer(size_t n) {
    if (n > pinnedCount_) {
        if (pinned_) PE_CHECK(cudaFreeHost(pinned_));
        pinned_ = nullptr;
        PE_CHECK(cudaMallocHost(&pinned_, n * sizeof(float4)));
        pinnedCount_ = n;
    }
    return pinned_;
}

void World::writeForces(const float *forces, uint32_t n) {
    PE_CHECK(cudaSetDevice(device_));
    if (hostDirty_) {
        pull();
        push();
    }
    stageForces(forces, n);
    PE_CHECK(cudaStreamSynchronize(stream_));  // the caller may reuse its array on return
}

// Caller forces copied as they are and expanded on the device (static and dead
// bodies masked); enqueued only: the caller's array must stay valid until the
// stream is next synchronised.
void World::stageForces(const float *forces, uint32_t n) {
    n = std::min<uint32_t>(n, nb_);
    if (n) {
        // the caller's array as it is; static and dead bodies masked on the device
        xfer3_.reserve(3 * (size_t)nb_);
        PE_CHECK(cudaMemcpyAsync(xfer3_.ptr, forces, 3 * (size_t)n * sizeof(float), cudaMemcpyHostToDevice, stream_));
        // a nonzero force wakes its body (RigidBody::applyForce)
        launchExpandForces(xfer3_.ptr, bflags_.ptr, force_.ptr, n, stream_,
                           sleepingEnabled ? sleep_[cur_].ptr : nullptr);
        if (sleepingEnabled) {
            wakeCheck_ = true;
            // keep a current host mirror current (a stale one is refreshed
            // from the device flags at its next pull)
            if (!deviceNewer_)
                for (uint32_t i = 0; i < n; ++i) {
                    HostBody &b = bodies[i];
                    if (b.alive && !b.isStatic &&
                        (forces[3 * i] != 0.0f || forces[3 * i + 1] != 0.0f || forces[3 * i + 2] != 0.0f))
                        b.wakeUp();
                }
        }
    }
    forces_ = true;
}

void World::readPoses(float *positions, float *rotations) {
    PE_CHECK(cudaSetDevice(device_));
    if (hostDirty_) {
        pull();
        push();
    }
    if (nb_) {
        enqueuePoses(cur_, positions, rotations);
        PE_CHECK(cudaStreamSynchronize(stream_));
    }
}

// Positions packed to the caller's 3 floats on the device (rotations are
// already 4 floats per body) from state copy `which`; enqueued only.
void World::enqueuePoses(int which, float *positions, float *rotations) {
    if (positions) {
        xfer3_.reserve(3 * (size_t)nb_);
        launchPackPositions(pos_[which].ptr, xfer3_.ptr, nb_, stream_);
        PE_CHECK(cudaMemcpyAsync(positions, xfer3_.ptr, 3 * (size_t)nb_ * sizeof(float), cudaMemcpyDeviceToHost,
                                 stream_));
    }
    if (rotations)
        PE_CHECK(cudaMemcpyAsync(rotations, rot_[which].ptr, (size_t)nb_ * sizeof(float4), cudaMemcpyDeviceToHost,
                                 stream_));
}

// ------------------------------------------------------------- downloads ---
void World::downloadPairs(uint32_t *pairs) {
    std::vector<uint32_t> a(lastPairs_), b(lastPairs_);
    if (lastPairs_) {
        PE_CHECK(cudaMemcpy(a.data(), pairA_.ptr, lastPairs_ * 4, cudaMemcpyDeviceToHost));
        PE_CHECK(cudaMemcpy(b.data(), pairB_.ptr, lastPairs_ * 4, cudaMemcpyDeviceToHost));
    }
    for (uint32_t i = 0; i < lastPairs_; ++i) {
        pairs[2 * i] = a[i];
        pairs[2 * i + 1] = b[i];
    }
}

struct ManifoldRecord {
    uint32_t aIdx, aGen, bIdx, bGen;
    float normal[3];
    uint32_t pointCount;
    float friction, restitution;
    float anchorA[4][3];
    float anchorB[4][3];
    float penetration[4];
    float normalImpulse[4];
    float tangentImpulse1[4];
    float tangentImpulse2[4];
    uint32_t feature[4];
};
static_assert(sizeof(ManifoldRecord) == 216, "manifold record layout");

void downloadManifoldRecords(const ManifoldView &mv, uint32_t M, void *records) {
    std::vector<uint32_t> ba(M), ga(M), bbv(M), gb(M), cnt(M), feat(4 * (size_t)M);
    std::vector<float4> nf(M), aa(4 * (size_t)M), ab(4 * (size_t)M), im(4 * (size_t)M);
    std::vector<float> rest(M);
    if (M) {
        PE_CHECK(cudaMemcpy(ba.data(), mv.bodyA, M * 4, cudaMemcpyDeviceToHost));
        PE_CHECK(cudaMemcpy(ga.data(), mv.genA, M * 4, cudaMemcpyDeviceToHost));
        PE_CHECK(cudaMemcpy(bbv.data(), mv.bodyB, M * 4, cudaMemcpyDeviceToHost));
        PE_CHECK(cudaMemcpy(gb.data(), mv.genB, M * 4, cudaMemcpyDeviceToHost));
        PE_CHECK(cudaMemcpy(cnt.data(), mv.pointCount, M * 4, cudaMemcpyDeviceToHost));
        PE_CHECK(cudaMemcpy(feat.data(), mv.feature, 4 * (size_t)M * 4, cudaMemcpyDeviceToHost));
        PE_CHECK(cudaMemcpy(nf.data(), mv.normalFriction, M * sizeof(float4), cudaMemcpyDeviceToHost));
        PE_CHECK(cudaMemcpy(aa.data(), mv.anchorA, 4 * (size_t)M * sizeof(float4), cudaMemcpyDeviceToHost));
        PE_CHECK(cudaMemcpy(ab.data(), mv.anchorB, 4 * (size_t)M * sizeof(float4), cudaMemcpyDeviceToHost));
        PE_CHECK(cudaMemcpy(im.data(), mv.impulse, 4 * (size_t)M * sizeof(float4), cudaMemcpyDeviceToHost));
        PE_CHECK(cudaMemcpy(rest.data(), mv.restitution, M * 4, cudaMemcpyDeviceToHost));
    }
    ManifoldRecord *out = (ManifoldRecord *)records;
    for (uint32_t m = 0; m < M; ++m) {
        ManifoldRecord &r = out[m];
        std::memset(&r, 0, sizeof(r));
        r.aIdx = ba[m];
        r.aGen = ga[m];
        r.bIdx = bbv[m];
        r.bGen = gb[m];
        r.normal[0] = nf[m].x;
        r.normal[1] = nf[m].y;
        r.normal[2] = nf[m].z;
        r.friction = nf[m].w;
        r.restitution = rest[m];
        r.pointCount = cnt[m];
        for (int k = 0; k < 4; ++k) {
            const float4 &A = aa[4 * m + k], &B = ab[4 * m + k], &I = im[4 * m + k];
            r.anchorA[k][0] = A.x; r.anchorA[k][1] = A.y; r.anchorA[k][2] = A.z;
            r.anchorB[k][0] = B.x; r.anchorB[k][1] = B.y; r.anchorB[k][2] = B.z;
            r.penetration[k] = A.w;
            r.normalImpulse[k] = I.x;
            r.tangentImpulse1[k] = I.y;
            r.tangentImpulse2[k] = I.z;
            r.feature[k] = feat[4 * m + k];
        }
    }
}

void World::downloadManifolds(void *records, uint32_t count) {
    downloadManifoldRecords(manifoldView(), std::min(count, lastManifolds_), records);
}

void World::downloadOrder(uint32_t *order, uint32_t *colors) {
    const uint32_t M = lastManifolds_;
    if (!M) return;
    if (orderMode == 0) {
        for (uint32_t m = 0; m < M; ++m) {
            if (order) order[m] = m;
            if (colors) colors[m] = m;
        }
        return;
    }
    // The solve order is (colour, manifold index); the island solver does not
    // materialise it, so it is derived from the colours here.
    std::vector<uint32_t> c(M, 0u);
    if (!solveSkipped_) PE_CHECK(cudaMemcpy(c.data(), sColor_.ptr, M * 4, cudaMemcpyDeviceToHost));
    if (colors) std::memcpy(colors, c.data(), M * 4);
    if (order) {
        uint32_t C = 0;
        for (uint32_t v : c) C = std::max(C, v + 1);
        std::vector<uint32_t> start(C + 1, 0);
        for (uint32_t v : c) ++start[v + 1];
        for (uint32_t k = 0; k < C; ++k) start[k + 1] += start[k];
        for (uint32_t m = 0; m < M; ++m) order[start[c[m]]++] = m;
    }
}

// --------------------------------------------------------------- stages ----
void World::broadphaseOnly(const float *mins, const float *maxs, uint32_t n, int algo, double cell,
                           std::vector<uint32_t> &pairs, StepCounters &c) {
    PE_CHECK(cudaSetDevice(device_));
    if (algo == 2) throw std::invalid_argument("DynamicTree requires a persistent DynamicAabbTree instance");
    uint32_t saveNc = nc_;
    nc_ = std::max(nc_, n);
    ensureCapacity();
    nc_ = saveNc;
    std::vector<float4> mn(n), mx(n);
    std::vector<uint32_t> keys(n), vals(n);
    for (uint32_t i = 0; i < n; ++i) {
        mn[i] = make_float4(mins[3 * i], mins[3 * i + 1], mins[3 * i + 2], 0.0f);
        mx[i] = make_float4(maxs[3 * i], maxs[3 * i + 1], maxs[3 * i + 2], 0.0f);
    }
    for (int attempt = 0; attempt < 8; ++attempt) {
        cudaStream_t s = stream_;
        DevStats *st = stats_.ptr;
        if (n) {
            PE_CHECK(cudaMemcpyAsync(inMin_.ptr, mn.data(), n * sizeof(float4), cudaMemcpyHostToDevice, s));
            PE_CHECK(cudaMemcpyAsync(inMax_.ptr, mx.data(), n * sizeof(float4), cudaMemcpyHostToDevice, s));
        }
        launchStepInit(st, n, s);
        BroadInput in{inMin_.ptr, inMax_.ptr, &st->inputCount, std::max<uint32_t>(n, 1)};
        uint32_t bits = 1;
        while (bits < 32 && (1ull << bits) < (unsigned long long)std::max<uint32_t>(n, 2)) ++bits;
        pb_.bits = bits;
        pb_.blockPath = false;
        pb_.bodyPath = false;
        bb_.hashed = false;
        bb_.keyBits = 64;
        if (algo == 0) {
            launchSapKeys(in, sapKeys_.ptr, sapVals_.ptr, s);
            launchSap(in, sapKeys_.ptr, sapVals_.ptr, bb_, pb_, st, ws_, s);
        } else {
            launchGrid(in, cell, bb_, pb_, st, ws_, s);
        }
        launchPairsFinalize(nullptr, nullptr, nullptr, pb_, st, ws_, s);
        PE_CHECK(cudaMemcpyAsync(hostStats_, st, sizeof(DevStats), cudaMemcpyDeviceToHost, s));
        PE_CHECK(cudaStreamSynchronize(s));
        const DevStats &h = *hostStats_;
        if (h.err & (kErrTimeout | kErrEntryCapacity)) throw std::runtime_error("broadphase failed on the device");
        bool retry = false;
        if (h.rawPairs > pairCap_) {
            pairCap_ = grow(h.rawPairs, pairCap_);
            retry = true;
        }
        if (h.gridEntryCount > entryCap_) {
            entryCap_ = grow(h.gridEntryCount, entryCap_);
            retry = true;
        }
        if (retry) {
            uint32_t save = nc_;
            nc_ = std::max(nc_, n);
            ensureCapacity();
            nc_ = save;
            continue;
        }
        c = StepCounters{};
        c.xWindow = algo == 0 ? h.xWindow : 0;
        c.aabbPairs = h.uniquePairs;
        c.gridComparisons = h.gridComparisons;
        c.gridEntries = algo == 1 ? h.gridEntryCount : 0;
        c.gridOverflow = algo == 1 ? h.overflowCount : 0;
        c.cellSize = algo == 1 ? h.cellSize : 0.0;
        pairs.resize(2 * (size_t)h.pairs);
        std::vector<uint32_t> a(h.pairs), b(h.pairs);
        if (h.pairs) {
            PE_CHECK(cudaMemcpy(a.data(), pairA_.ptr, h.pairs * 4, cudaMemcpyDeviceToHost));
            PE_CHECK(cudaMemcpy(b.data(), pairB_.ptr, h.pairs * 4, cudaMemcpyDeviceToHost));
        }
        for (uint32_t i = 0; i < h.pairs; ++i) {
            pairs[2 * i] = a[i];
            pairs[2 * i + 1] = b[i];
        }
        return;
    }
    throw std::runtime_error("broadphase buffers kept overflowing");
}

void World::solveOnly(std::vector<float> &recs, uint32_t count, float dt, int iters, int mode) {
    PE_CHECK(cudaSetDevice(device_));
    if (hostDirty_) {
        pull();
        push();
    }
    if (count > mcap_) {
        mcap_ = grow(count, mcap_);
        ensureCapacity();
    }
    ManifoldRecord *r = (ManifoldRecord *)recs.data();
    std::vector<uint32_t> ba(count), ga(count), bbv(count), gb(count), cnt(count), feat(4 * (size_t)count);
    std::vector<float4> nf(count), aa(4 * (size_t)count), ab(4 * (size_t)count), im(4 * (size_t)count);
    std::vector<float> rest(count);
    for (uint32_t m = 0; m < count; ++m) {
        ba[m] = r[m].aIdx;
        ga[m] = r[m].aGen;
        bbv[m] = r[m].bIdx;
        gb[m] = r[m].bGen;
        // a ContactManifold holds at most four points (manifold.hpp:21-34)
        if (r[m].pointCount > 4) throw std::invalid_argument("a contact manifold holds at most 4 points");
        cnt[m] = r[m].pointCount;
        nf[m] = make_float4(r[m].normal[0], r[m].normal[1], r[m].normal[2], r[m].friction);
        rest[m] = r[m].restitution;
        for (int k = 0; k < 4; ++k) {
            aa[4 * m + k] = make_float4(r[m].anchorA[k][0], r[m].anchorA[k][1], r[m].anchorA[k][2], r[m].penetration[k]);
            ab[4 * m + k] = make_float4(r[m].anchorB[k][0], r[m].anchorB[k][1], r[m].anchorB[k][2], 0.0f);
            im[4 * m + k] = make_float4(r[m].normalImpulse[k], r[m].tangentImpulse1[k], r[m].tangentImpulse2[k], 0.0f);
            feat[4 * m + k] = r[m].feature[k];
        }
    }
    cudaStream_t s = stream_;
    auto up = [&](void *d, const void *h, size_t bytes) {
        if (bytes) PE_CHECK(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, s));
    };
    up(mBodyA_.ptr, ba.data(), count * 4);
    up(mGenA_.ptr, ga.data(), count * 4);
    up(mBodyB_.ptr, bbv.data(), count * 4);
    up(mGenB_.ptr, gb.data(), count * 4);
    up(mCount_.ptr, cnt.data(), count * 4);
    up(mFeature_.ptr, feat.data(), 4 * (size_t)count * 4);
    up(mNormal_.ptr, nf.data(), count * sizeof(float4));
    up(mAnchorA_.ptr, aa.data(), 4 * (size_t)count * sizeof(float4));
    up(mAnchorB_.ptr, ab.data(), 4 * (size_t)count * sizeof(float4));
    up(mImpulse_.ptr, im.data(), 4 * (size_t)count * sizeof(float4));
    up(mRest_.ptr, rest.data(), count * 4);
    DevStats *st = stats_.ptr;
    launchStepInit(st, 0, s);
    launchSetManifoldCount(st, count, s);
    const size_t bytes = (size_t)std::max<uint32_t>(nb_, 1) * sizeof(float4);
    PE_CHECK(cudaMemcpyAsync(pos_[1 - cur_].ptr, pos_[cur_].ptr, bytes, cudaMemcpyDeviceToDevice, s));
    PE_CHECK(cudaMemcpyAsync(rot_[1 - cur_].ptr, rot_[cur_].ptr, bytes, cudaMemcpyDeviceToDevice, s));
    PE_CHECK(cudaMemcpyAsync(lin_[1 - cur_].ptr, lin_[cur_].ptr, bytes, cudaMemcpyDeviceToDevice, s));
    PE_CHECK(cudaMemcpyAsync(ang_[1 - cur_].ptr, ang_[cur_].ptr, bytes, cudaMemcpyDeviceToDevice, s));
    WorldView w = view(dt);
    ManifoldView mv = manifoldView();
    uint32_t want = (count + 1023) / 1024, blocks = 1;
    while (blocks < want) blocks <<= 1;
    blocks = std::min<uint32_t>(blocks, (uint32_t)maxCooperativeBlocks(smCount_));
    const bool block = count <= kBlockMaxManifolds && nb_ <= kBlockMaxBodies;
    const bool sleeping = sleepingEnabled;
    const CacheView tmp{tKey_.ptr, tGens_.ptr, tA_.ptr, tB_.ptr, tT2_.ptr};
    if (sleeping) {
        // the sleep state is carried over unchanged; the solver's sleeping bit
        // comes from the committed flags
        const size_t n = std::max<uint32_t>(nb_, 1);
        PE_CHECK(cudaMemcpyAsync(sleep_[1 - cur_].ptr, sleep_[cur_].ptr, n * 4, cudaMemcpyDeviceToDevice, s));
        PE_CHECK(cudaMemcpyAsync(quiet_[1 - cur_].ptr, quiet_[cur_].ptr, n * 4, cudaMemcpyDeviceToDevice, s));
        launchSleepBits(w, sleep_[cur_].ptr, bflags_.ptr, st, s);
    }
    launchSolver(w, mv, cacheView(cache_), &cCount_.ptr[cache_], sleeping ? tmp : cacheView(1 - cache_),
                 sleeping ? tCount_.ptr : &cCount_.ptr[1 - cache_], cacheCap_, sb_, iters, mode, (int)blocks, block, 0u,
                 false, st, ws_, s);
    if (sleeping)
        launchCacheCarry(w, cacheView(cache_), &cCount_.ptr[cache_], tmp, tCount_.ptr, cacheView(1 - cache_),
                         &cCount_.ptr[1 - cache_], cacheCap_, carry_.ptr, carryPos_.ptr, carryTotal_.ptr, st, ws_, s);
    PE_CHECK(cudaMemcpyAsync(hostStats_, st, sizeof(DevStats), cudaMemcpyDeviceToHost, s));
    PE_CHECK(cudaStreamSynchronize(s));
    if (hostStats_->err & (kErrTimeout | kErrColors | kErrCacheCapacity))
        throw std::runtime_error("solve failed on the device");
    counters_ = StepCounters{};
    counters_.solvedContactCount = hostStats_->solved;
    counters_.preparedPoints = hostStats_->preparedPoints;
    counters_.warmComparisons = hostStats_->warmComparisons;
    counters_.warmMatches = hostStats_->warmMatches;
    counters_.velocityPointVisits = hostStats_->preparedPoints * (uint64_t)iters;
    solveSkipped_ = sleepingEnabled && hostStats_->solveCount == 0;
    counters_.colors = mode == 0 ? count : solveSkipped_ ? (count ? 1u : 0u) : hostStats_->colors;
    cur_ = 1 - cur_;
    cache_ = 1 - cache_;
    deviceNewer_ = true;
    lastManifolds_ = count;
    downloadManifolds(recs.data(), count);
}

} // namespace pe
