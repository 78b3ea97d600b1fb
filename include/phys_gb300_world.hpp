// Header-only C++ facade with the public surface of bkuangs/phys-engine's
// phys::PhysicsWorld (include/phys/world/physics_world.hpp:21-153) over the C ABI
// in phys_gb300.h.  A caller of the reference switches by including this header,
// using namespace phys_gb300 instead of phys, and linking libphys_gb300.so.
//
// Differences a caller can see:
//   * getBody() returns a BodyRef (a handle-bound accessor with the RigidBody
//     member functions) instead of RigidBody*; it converts to false when the
//     handle is stale, where the reference returns nullptr.
//   * contacts() returns the manifolds by value (downloaded from the device).
//   * copies and moves are supported like the reference's; a moved-from world
//     holds no device world.
//   * colliders are added with addSphereCollider / addBoxCollider (the
//     reference's addCollider takes a Collider struct with a shape variant).
//   * solver iterations and order are configurable (the reference fixes 8 and
//     manifold order); the default here is the reference's 8 with the GPU's
//     graph-colour order.
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "phys_gb300.h"

namespace phys_gb300 {

struct Vec3 {
    float x{}, y{}, z{};
};
struct Quaternion {
    float x{}, y{}, z{}, w{1.0f};
};
struct RigidBodyHandle {
    uint32_t index = 0;
    uint32_t generation = 0;
};
struct ColliderHandle {
    uint32_t index = 0;
    uint32_t generation = 0;
};
enum class BroadPhaseAlgorithm { SweepAndPrune, UniformGrid, DynamicTree };

struct ContactPoint {
    Vec3 localAnchorA{};
    Vec3 localAnchorB{};
    float penetration = 0.0f;
    float normalImpulse = 0.0f;
    float tangentImpulse1 = 0.0f;
    float tangentImpulse2 = 0.0f;
    uint32_t feature = 0;
};
struct ContactManifold {
    RigidBodyHandle bodyA{};
    RigidBodyHandle bodyB{};
    Vec3 normal{};
    ContactPoint points[4]{};
    uint32_t pointCount = 0;
    float friction = 0.0f;
    float restitution = 0.0f;
};
using StepStats = pe_step_stats;

inline void throwIf(pe_status s) {
    if (s == PE_OK) return;
    if (s == PE_ERR_INVALID_ARGUMENT || s == PE_ERR_UNSUPPORTED) throw std::invalid_argument(pe_last_error());
    throw std::runtime_error(pe_last_error());
}

class PhysicsWorld;

// RigidBody accessor (include/phys/dynamics/rigid_body.hpp:14-140) bound to a handle.
class BodyRef {
  public:
    explicit operator bool() const { return ok_; }
    Vec3 getPosition() const { return {s_.position[0], s_.position[1], s_.position[2]}; }
    Quaternion getRotation() const { return {s_.rotation[0], s_.rotation[1], s_.rotation[2], s_.rotation[3]}; }
    Vec3 getLinearVelocity() const { return {s_.linear_velocity[0], s_.linear_velocity[1], s_.linear_velocity[2]}; }
    Vec3 getAngularVelocity() const {
        return {s_.angular_velocity[0], s_.angular_velocity[1], s_.angular_velocity[2]};
    }
    float mass() const { return s_.mass; }
    float restitution() const { return s_.restitution; }
    float friction() const { return s_.friction; }
    bool isStatic() const { return s_.is_static != 0; }
    float getInverseMass() const { return isStatic() || s_.mass <= 0.0f ? 0.0f : 1.0f / s_.mass; }
    // The velocity setters, applyForce and applyLinearImpulse wake the body
    // like the reference's (rigid_body.hpp:54-95).
    bool isSleeping() const {
        int v = 0;
        if (ok_) throwIf(pe_world_body_is_sleeping(w_, h_, &v));
        return v != 0;
    }
    void wakeUp() {
        if (ok_) throwIf(pe_world_body_wake_up(w_, h_));
    }
    void setLinearVelocity(const Vec3 &v) {
        const float l[3] = {v.x, v.y, v.z};
        if (ok_) throwIf(pe_world_body_set_velocity(w_, h_, l, nullptr));
        refresh();
    }
    void setAngularVelocity(const Vec3 &v) {
        const float a[3] = {v.x, v.y, v.z};
        if (ok_) throwIf(pe_world_body_set_velocity(w_, h_, nullptr, a));
        refresh();
    }
    void applyForce(const Vec3 &f) {
        const float v[3] = {f.x, f.y, f.z};
        if (ok_) throwIf(pe_world_body_apply_force(w_, h_, v));
        refresh();
    }
    void applyLinearImpulse(const Vec3 &j) {
        if (isStatic() || (j.x == 0.0f && j.y == 0.0f && j.z == 0.0f)) return;
        const float m = getInverseMass();
        setLinearVelocity({s_.linear_velocity[0] + j.x * m, s_.linear_velocity[1] + j.y * m,
                           s_.linear_velocity[2] + j.z * m});
    }
    void clearForces() {
        s_.force[0] = s_.force[1] = s_.force[2] = 0.0f;
        commit();
    }
    void setMass(float m) {
        s_.mass = m;
        commit();
    }
    void setStatic(bool st) {
        s_.is_static = st ? 1 : 0;
        commit();
    }
    void integrateRotation(float dt) {
        throwIf(pe_world_body_integrate_rotation(w_, h_, dt));
        refresh();
    }

  private:
    friend class PhysicsWorld;
    BodyRef(pe_world *w, RigidBodyHandle h) : w_(w), h_{h.index, h.generation} { refresh(); }
    void refresh() { ok_ = pe_world_get_body(w_, h_, &s_) == PE_OK; }
    void commit() {
        if (ok_) throwIf(pe_world_set_body(w_, h_, &s_));
    }
    pe_world *w_;
    pe_handle h_;
    pe_body_state s_{};
    bool ok_ = false;
};

class PhysicsWorld {
  public:
    static constexpr float minBodySize = 0.01f * 0.01f;
    static constexpr float maxBodySize = 64.0f * 64.0f;
    static constexpr float minDensity = 0.2f;
    static constexpr float maxDensity = 21.4f;

    Vec3 gravity{0.0f, -9.81f, 0.0f};
    BroadPhaseAlgorithm broadPhaseAlgorithm = BroadPhaseAlgorithm::SweepAndPrune;

    explicit PhysicsWorld(int device = 0, int solverIterations = 8, int order = PE_ORDER_COLOR) {
        throwIf(pe_world_create(device, &w_));
        throwIf(pe_world_set_solver(w_, solverIterations, order));
    }
    ~PhysicsWorld() {
        if (w_) pe_world_destroy(w_);
    }
    // Copies are independent worlds with the same state (physics_world.cpp:74-120).
    PhysicsWorld(const PhysicsWorld &o)
        : gravity(o.gravity), broadPhaseAlgorithm(o.broadPhaseAlgorithm), npWorkers_(o.npWorkers_),
          solverWorkers_(o.solverWorkers_), broadWorkers_(o.broadWorkers_) {
        throwIf(pe_world_clone(o.w_, &w_));
    }
    PhysicsWorld &operator=(const PhysicsWorld &o) {
        if (this == &o) return *this;
        pe_world *c = nullptr;
        throwIf(pe_world_clone(o.w_, &c));
        if (w_) pe_world_destroy(w_);
        w_ = c;
        gravity = o.gravity;
        broadPhaseAlgorithm = o.broadPhaseAlgorithm;
        npWorkers_ = o.npWorkers_;
        solverWorkers_ = o.solverWorkers_;
        broadWorkers_ = o.broadWorkers_;
        return *this;
    }
    PhysicsWorld(PhysicsWorld &&o) noexcept
        : gravity(o.gravity), broadPhaseAlgorithm(o.broadPhaseAlgorithm), w_(o.w_), npWorkers_(o.npWorkers_),
          solverWorkers_(o.solverWorkers_), broadWorkers_(o.broadWorkers_) {
        o.w_ = nullptr;
    }
    PhysicsWorld &operator=(PhysicsWorld &&o) noexcept {
        if (this == &o) return *this;
        if (w_) pe_world_destroy(w_);
        w_ = o.w_;
        o.w_ = nullptr;
        gravity = o.gravity;
        broadPhaseAlgorithm = o.broadPhaseAlgorithm;
        npWorkers_ = o.npWorkers_;
        solverWorkers_ = o.solverWorkers_;
        broadWorkers_ = o.broadWorkers_;
        return *this;
    }

    bool createSphere(float radius, Vec3 position, float density, bool isStatic, float restitution, float friction,
                      RigidBodyHandle &body, ColliderHandle &collider, std::string &errorMessage) {
        errorMessage.clear();
        float p[3] = {position.x, position.y, position.z};
        pe_handle b{}, c{};
        pe_status s = pe_world_create_sphere(w_, radius, p, density, isStatic, restitution, friction, &b, &c);
        return finishCreate(s, b, c, body, collider, errorMessage);
    }
    bool createBox(float width, float height, float depth, Vec3 position, float density, bool isStatic,
                   float restitution, float friction, RigidBodyHandle &body, ColliderHandle &collider,
                   std::string &errorMessage) {
        errorMessage.clear();
        float p[3] = {position.x, position.y, position.z};
        pe_handle b{}, c{};
        pe_status s = pe_world_create_box(w_, width, height, depth, p, density, isStatic, restitution, friction, &b, &c);
        return finishCreate(s, b, c, body, collider, errorMessage);
    }
    void removeBody(RigidBodyHandle h) { throwIf(pe_world_remove_body(w_, pe_handle{h.index, h.generation})); }
    void removeCollider(ColliderHandle h) { throwIf(pe_world_remove_collider(w_, pe_handle{h.index, h.generation})); }
    // addCollider (physics_world.hpp:57) with a sphere or box shape at a local
    // transform; an empty handle for a stale body, like the reference.
    ColliderHandle addSphereCollider(RigidBodyHandle body, float radius, Vec3 localPosition = {},
                                     Quaternion localRotation = {}) {
        const float d[3] = {radius, 0.0f, 0.0f};
        return addCollider(body, PE_SHAPE_SPHERE, d, localPosition, localRotation);
    }
    ColliderHandle addBoxCollider(RigidBodyHandle body, Vec3 halfExtents, Vec3 localPosition = {},
                                  Quaternion localRotation = {}) {
        const float d[3] = {halfExtents.x, halfExtents.y, halfExtents.z};
        return addCollider(body, PE_SHAPE_BOX, d, localPosition, localRotation);
    }
    BodyRef getBody(RigidBodyHandle h) { return BodyRef(w_, h); }

    void setNarrowPhaseWorkerCount(std::size_t n) { setWorkers(n, solverWorkers_, broadWorkers_, &npWorkers_); }
    void setSolverWorkerCount(std::size_t n) { setWorkers(npWorkers_, n, broadWorkers_, &solverWorkers_); }
    void setBroadPhaseWorkerCount(std::size_t n) { setWorkers(npWorkers_, solverWorkers_, n, &broadWorkers_); }
    std::size_t getNarrowPhaseWorkerCount() const { return npWorkers_; }
    std::size_t getSolverWorkerCount() const { return solverWorkers_; }
    std::size_t getBroadPhaseWorkerCount() const { return broadWorkers_; }
    void setSleepingEnabled(bool enabled) { throwIf(pe_world_set_sleeping_enabled(w_, enabled)); }
    bool isSleepingEnabled() const {
        int v = 0;
        throwIf(pe_world_get_sleeping_enabled(w_, &v));
        return v != 0;
    }

    void step(float dt) {
        throwIf(pe_world_set_gravity(w_, gravity.x, gravity.y, gravity.z));
        throwIf(pe_world_set_broadphase(w_, broadPhaseAlgorithm == BroadPhaseAlgorithm::UniformGrid ? PE_BROADPHASE_GRID
                                            : broadPhaseAlgorithm == BroadPhaseAlgorithm::DynamicTree ? PE_BROADPHASE_TREE
                                                                                                       : PE_BROADPHASE_SAP));
        throwIf(pe_world_step(w_, dt));
    }

    std::vector<ContactManifold> contacts() const {
        uint32_t n = 0;
        pe_status s = pe_world_get_contacts(w_, nullptr, 0, &n);
        if (s != PE_OK && s != PE_ERR_CAPACITY) throwIf(s);
        std::vector<pe_contact_manifold> raw(n);
        if (n) throwIf(pe_world_get_contacts(w_, raw.data(), n, &n));
        std::vector<ContactManifold> out(n);
        for (uint32_t m = 0; m < n; ++m) {
            const pe_contact_manifold &r = raw[m];
            ContactManifold &c = out[m];
            c.bodyA = {r.body_a_index, r.body_a_generation};
            c.bodyB = {r.body_b_index, r.body_b_generation};
            c.normal = {r.normal[0], r.normal[1], r.normal[2]};
            c.pointCount = r.point_count;
            c.friction = r.friction;
            c.restitution = r.restitution;
            for (int k = 0; k < 4; ++k) {
                c.points[k].localAnchorA = {r.anchor_a[k][0], r.anchor_a[k][1], r.anchor_a[k][2]};
                c.points[k].localAnchorB = {r.anchor_b[k][0], r.anchor_b[k][1], r.anchor_b[k][2]};
                c.points[k].penetration = r.penetration[k];
                c.points[k].normalImpulse = r.normal_impulse[k];
                c.points[k].tangentImpulse1 = r.tangent_impulse1[k];
                c.points[k].tangentImpulse2 = r.tangent_impulse2[k];
                c.points[k].feature = r.feature[k];
            }
        }
        return out;
    }

    StepStats lastStepStats() const {
        StepStats s{};
        throwIf(pe_world_get_step_stats(w_, &s));
        return s;
    }

    pe_world *native() const { return w_; }

  private:
    ColliderHandle addCollider(RigidBodyHandle body, int shape, const float *dims, Vec3 lp, Quaternion lq) {
        const float p[3] = {lp.x, lp.y, lp.z}, q[4] = {lq.x, lq.y, lq.z, lq.w};
        pe_handle c{};
        pe_status s = pe_world_add_collider(w_, pe_handle{body.index, body.generation}, shape, dims, p, q, &c);
        if (s == PE_ERR_STALE_HANDLE) return {};
        throwIf(s);
        return {c.index, c.generation};
    }
    bool finishCreate(pe_status s, pe_handle b, pe_handle c, RigidBodyHandle &body, ColliderHandle &collider,
                      std::string &errorMessage) {
        if (s == PE_ERR_CREATE_FAILED) {
            errorMessage = pe_last_error();
            return false;
        }
        throwIf(s);
        body = {b.index, b.generation};
        collider = {c.index, c.generation};
        return true;
    }
    void setWorkers(std::size_t np, std::size_t solver, std::size_t bp, std::size_t *which) {
        throwIf(pe_world_set_worker_counts(w_, np, solver, bp));
        *which = which == &npWorkers_ ? np : which == &solverWorkers_ ? solver : bp;
    }
    pe_world *w_ = nullptr;
    std::size_t npWorkers_ = 1, solverWorkers_ = 1, broadWorkers_ = 1;
};

} // namespace phys_gb300
