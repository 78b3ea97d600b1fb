// Header-only C++ facade with the public surface of bkuangs/phys-engine's
// phys::PhysicsWorld and the types its callers touch, over the C ABI in
// phys_gb300.h:
//   include/phys/world/physics_world.hpp:21-77     PhysicsWorld
//   include/phys/dynamics/rigid_body.hpp:14-140    RigidBody
//   include/phys/collision/collider.hpp:12-31      Collider, ColliderHandle
//   include/phys/collision/broadphase.hpp:8-55     BroadPhase, BroadPhasePair, BroadPhaseStats
//   include/phys/collision/narrowphase.hpp:10-40   NarrowPhase
//   include/phys/solver/sequential_impulse_solver.hpp:14-17  SequentialImpulseSolver::solve
//   include/phys/collision/manifold.hpp:9-34       ContactPoint, ContactManifold
//   include/phys/world/step_stats.hpp:7-54         StepStats
//   include/phys/math/*.hpp                        Vec3, Quaternion, Mat3, Transform, Math3d
// A caller of the reference switches by including this header, writing
// `namespace phys = phys_gb300;` (or using phys_gb300:: names) and linking
// libphys_gb300.so.  The public types keep the reference's names, members and
// signatures so that code written against phys:: compiles unchanged.
//
// What differs underneath:
//   * The world lives on the GPU.  getBody() / getCollider() return pointers to
//     host copies owned by the world object, fetched on the call; edits made
//     through them are written back at the world's next call (step, solve,
//     another getBody, ...).  The reference says such a pointer is for
//     immediate work only (physics_world.hpp:52-55), which is exactly the
//     window in which these copies are current.
//   * contacts() and lastStepStats() are read back from the device on first
//     use after a step.
//   * The default constructor solves in the reference's manifold order
//     (PE_ORDER_MANIFOLD: results equal the reference's bit for bit); pass
//     PE_ORDER_COLOR to solve in the GPU's parallel graph-colour order.
//   * Solver iterations are configurable (the reference fixes 8).
//   * BroadPhase / NarrowPhase statics run on GPU device 0 (setDevice changes it).
#pragma once
#include <array>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <utility>
#include <variant>
#include <vector>

#include "phys_gb300.h"

namespace phys_gb300 {

inline void throwIf(pe_status s) {
    if (s == PE_OK) return;
    if (s == PE_ERR_INVALID_ARGUMENT || s == PE_ERR_UNSUPPORTED) throw std::invalid_argument(pe_last_error());
    throw std::runtime_error(pe_last_error());
}

// ------------------------------------------------------------------ math ---
struct MathConstants {
    static constexpr float pi = 3.14159265358979323846f;
};
struct BodyLimits {
    static constexpr float minSize = 0.01f * 0.01f;
    static constexpr float maxSize = 64.0f * 64.0f;
    static constexpr float minDensity = 0.2f;
    static constexpr float maxDensity = 21.4f;
};

struct Vec3 {
    float x{}, y{}, z{};
    Vec3 &operator+=(const Vec3 &o) {
        x += o.x;
        y += o.y;
        z += o.z;
        return *this;
    }
    Vec3 &operator-=(const Vec3 &o) {
        x -= o.x;
        y -= o.y;
        z -= o.z;
        return *this;
    }
    Vec3 operator-() const { return {-x, -y, -z}; }
    static constexpr Vec3 zero() { return {0.0f, 0.0f, 0.0f}; }
};
inline Vec3 operator+(Vec3 a, const Vec3 &b) { return a += b; }
inline Vec3 operator-(Vec3 a, const Vec3 &b) { return a -= b; }
inline Vec3 operator*(Vec3 v, float s) { return {v.x * s, v.y * s, v.z * s}; }
inline Vec3 operator*(float s, Vec3 v) { return {s * v.x, s * v.y, s * v.z}; }
inline Vec3 operator/(Vec3 v, float s) { return {v.x / s, v.y / s, v.z / s}; }

struct Mat3 {
    float m00{}, m01{}, m02{};
    float m10{}, m11{}, m12{};
    float m20{}, m21{}, m22{};
    static Mat3 identity() { return {1.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 1.0f}; }
    Vec3 operator*(const Vec3 &v) const {
        return {m00 * v.x + m01 * v.y + m02 * v.z, m10 * v.x + m11 * v.y + m12 * v.z,
                m20 * v.x + m21 * v.y + m22 * v.z};
    }
    Mat3 &operator+=(const Mat3 &o) {
        m00 += o.m00, m01 += o.m01, m02 += o.m02;
        m10 += o.m10, m11 += o.m11, m12 += o.m12;
        m20 += o.m20, m21 += o.m21, m22 += o.m22;
        return *this;
    }
};
inline Mat3 operator+(Mat3 a, const Mat3 &b) { return a += b; }
inline Mat3 transpose(const Mat3 &m) { return {m.m00, m.m10, m.m20, m.m01, m.m11, m.m21, m.m02, m.m12, m.m22}; }
inline Mat3 operator*(const Mat3 &a, const Mat3 &b) {
    auto row = [&](float r0, float r1, float r2, int c) {
        const float b0 = c == 0 ? b.m00 : c == 1 ? b.m01 : b.m02;
        const float b1 = c == 0 ? b.m10 : c == 1 ? b.m11 : b.m12;
        const float b2 = c == 0 ? b.m20 : c == 1 ? b.m21 : b.m22;
        return r0 * b0 + r1 * b1 + r2 * b2;
    };
    return {row(a.m00, a.m01, a.m02, 0), row(a.m00, a.m01, a.m02, 1), row(a.m00, a.m01, a.m02, 2),
            row(a.m10, a.m11, a.m12, 0), row(a.m10, a.m11, a.m12, 1), row(a.m10, a.m11, a.m12, 2),
            row(a.m20, a.m21, a.m22, 0), row(a.m20, a.m21, a.m22, 1), row(a.m20, a.m21, a.m22, 2)};
}

struct Quaternion {
    float x{}, y{}, z{}, w{1.0f};
    static constexpr Quaternion identity() { return {0.0f, 0.0f, 0.0f, 1.0f}; }
    // axis of unit length, angle in radians
    static Quaternion fromAxisAngle(Vec3 axis, float angleRadians) {
        const float h = angleRadians * 0.5f, s = std::sin(h);
        return {axis.x * s, axis.y * s, axis.z * s, std::cos(h)};
    }
    // Hamilton product
    Quaternion operator*(const Quaternion &o) const {
        return {w * o.x + x * o.w + y * o.z - z * o.y, w * o.y - x * o.z + y * o.w + z * o.x,
                w * o.z + x * o.y - y * o.x + z * o.w, w * o.w - x * o.x - y * o.y - z * o.z};
    }
    Quaternion conjugate() const { return {-x, -y, -z, w}; }
    float length() const { return std::sqrt(x * x + y * y + z * z + w * w); }
    Quaternion normalized() const {
        const float n = length();
        if (n == 0.0f) return identity();
        return {x / n, y / n, z / n, w / n};
    }
    Vec3 rotate(const Vec3 &v) const {
        const Quaternion r = (*this) * Quaternion{v.x, v.y, v.z, 0.0f} * conjugate();
        return {r.x, r.y, r.z};
    }
    Mat3 toMat3() const {
        const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, xz = x * z, yz = y * z;
        const float wx = w * x, wy = w * y, wz = w * z;
        return {1.0f - 2.0f * (yy + zz), 2.0f * (xy - wz),        2.0f * (xz + wy),
                2.0f * (xy + wz),        1.0f - 2.0f * (xx + zz), 2.0f * (yz - wx),
                2.0f * (xz - wy),        2.0f * (yz + wx),        1.0f - 2.0f * (xx + yy)};
    }
};

struct Transform {
    Vec3 position{};
    Quaternion orientation = Quaternion::identity();
    constexpr Transform() = default;
    static constexpr Transform zero() { return {}; }
    Transform(Vec3 p, Quaternion q) : position(p), orientation(q) {}
    // rotation about z
    Transform(Vec3 p, float zAngleRadians)
        : position(p), orientation(Quaternion::fromAxisAngle({0.0f, 0.0f, 1.0f}, zAngleRadians)) {}
};
inline Vec3 transform(Vec3 v, const Transform &tf) { return tf.orientation.rotate(v) + tf.position; }

class Math3d {
  public:
    static float dot(Vec3 a, Vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
    static Vec3 cross(Vec3 a, Vec3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
    static float length(Vec3 v) { return std::sqrt(dot(v, v)); }
    static float distance(Vec3 a, Vec3 b) { return length(a - b); }
    // zero for lengths up to 1e-8, else v * (1 / |v|)
    static Vec3 normalize(Vec3 v) {
        const float n = length(v);
        if (n <= 1e-8f) return Vec3::zero();
        return v * (1.0f / n);
    }
    static float sin(float r) { return std::sin(r); }
    static float cos(float r) { return std::cos(r); }
    static float clamp(float value, float lo, float hi) {
        if (lo == hi) return lo;
        if (lo > hi) throw std::invalid_argument("clamp minimum exceeds maximum");
        return value < lo ? lo : value > hi ? hi : value;
    }
};

// --------------------------------------------------------------- handles ---
struct RigidBodyHandle {
    uint32_t index = 0;
    uint32_t generation = 0;
};
inline bool operator==(const RigidBodyHandle &a, const RigidBodyHandle &b) {
    return a.index == b.index && a.generation == b.generation;
}
struct ColliderHandle {
    uint32_t index = 0;
    uint32_t generation = 0;
};
inline bool operator==(const ColliderHandle &a, const ColliderHandle &b) {
    return a.index == b.index && a.generation == b.generation;
}

// ---------------------------------------------------------------- shapes ---
struct Sphere {
    float radius{};
};
struct Box {
    Vec3 halfExtents{};
};
struct Aabb {
    Vec3 min{};
    Vec3 max{};
    // closed intervals: touching boxes overlap
    bool overlaps(const Aabb &o) const {
        return min.x <= o.max.x && max.x >= o.min.x && min.y <= o.max.y && max.y >= o.min.y && min.z <= o.max.z &&
               max.z >= o.min.z;
    }
};
struct Collider {
    RigidBodyHandle body{};
    Transform localTransform{};
    std::variant<Sphere, Box> shape = Sphere{};
    Aabb bounds{};
};

// -------------------------------------------------------------- contacts ---
struct ContactPoint {
    Vec3 localAnchorA{};
    Vec3 localAnchorB{};
    float penetration = 0.0f;
    float normalImpulse = 0.0f;
    float tangentImpulse1 = 0.0f;
    float tangentImpulse2 = 0.0f;
    uint32_t feature = 0;  // added: (kind << 24) | (source << 16) | (face axis << 8) | (face sign << 4) | vertex
};
struct ContactManifold {
    RigidBodyHandle bodyA{};
    RigidBodyHandle bodyB{};
    Vec3 normal{};  // from body A toward body B
    std::array<ContactPoint, 4> points{};
    uint32_t pointCount = 0;
    float friction = 0.0f;
    float restitution = 0.0f;
};

enum class BroadPhaseAlgorithm { SweepAndPrune, UniformGrid, DynamicTree };
struct BroadPhasePair {
    std::size_t first;
    std::size_t second;
};
// Counters of the reference's BroadPhaseStats; the timings hold the device time
// of the whole broadphase stage in sweepMs, and the incremental tree's
// maintenance counters stay zero (the device rebuilds a linear BVH instead).
struct BroadPhaseStats {
    double recordBuildMs = 0.0, recordSortMs = 0.0, sweepMs = 0.0, pairSortMs = 0.0;
    std::size_t xWindowComparisons = 0, aabbPairs = 0, gridComparisons = 0, gridEntries = 0, gridOverflowAabbs = 0;
    double gridCellSize = 0.0;
    std::size_t treeInsertions = 0, treeRemovals = 0, treeReinsertions = 0, treeNodePairVisits = 0,
                treeLeafChecks = 0, treeHeight = 0, treeProxyCount = 0;
};
struct NarrowPhaseStats {
    std::size_t sphereSphereCandidates = 0, sphereBoxCandidates = 0, boxBoxCandidates = 0;
    std::size_t sphereSphereContacts = 0, sphereBoxContacts = 0, boxBoxContacts = 0;
};
struct SolverStats {
    double prepareMs = 0.0, warmStartMs = 0.0, velocityIterationsMs = 0.0, cacheUpdateMs = 0.0;
    std::size_t preparedPoints = 0, warmStartComparisons = 0, warmStartMatches = 0, velocityPointVisits = 0;
    std::size_t islandCount = 0, largestIslandContacts = 0, largestIslandPoints = 0;
};
// StepStats of the last step; stage times are device times of the GPU stages.
struct StepStats {
    double totalMs = 0.0, integrateVelocityMs = 0.0, broadPhaseMs = 0.0, narrowPhaseMs = 0.0, solverMs = 0.0,
           integratePoseMs = 0.0;
    double broadPhaseCollectMs = 0.0, broadPhaseFilterMs = 0.0;
    BroadPhaseStats broadPhaseDetails{};
    NarrowPhaseStats narrowPhaseDetails{};
    SolverStats solverDetails{};
    std::size_t possiblePairs = 0, candidatePairs = 0, contactCount = 0, solvedContactCount = 0;
    std::size_t awakeBodyCount = 0, sleepingBodyCount = 0;
};

class PhysicsWorld;
class SequentialImpulseSolver;

// ------------------------------------------------------------- RigidBody ---
class RigidBody {
  public:
    RigidBody() = default;
    float mass{};
    float restitution{};
    float friction{};
    bool isStatic{};
    RigidBody(Vec3 p, float m, float e, float mu, bool st)
        : mass(m), restitution(e), friction(mu), isStatic(st), position(p) {}

    void integratePosition(float dt) { integrate(PE_INTEGRATE_POSITION, nullptr, dt); }
    void integrateVelocity(const Vec3 &gravity, float dt) {
        const float g[3] = {gravity.x, gravity.y, gravity.z};
        integrate(PE_INTEGRATE_VELOCITY, g, dt);
    }
    void integrateRotation(float dt) { integrate(PE_INTEGRATE_ROTATION, nullptr, dt); }

    Vec3 getPosition() const { return position; }
    Vec3 getLinearVelocity() const { return linearVelocity; }
    bool isSleeping() const { return !isStatic && sleeping; }
    void wakeUp() {
        sleeping = false;
        wakeRequested = true;
    }
    void setLinearVelocity(const Vec3 &v) {
        wakeUp();
        linearVelocity = v;
    }
    void applyLinearImpulse(const Vec3 &j) {
        if (isStatic) return;
        if (j.x != 0.0f || j.y != 0.0f || j.z != 0.0f) wakeUp();
        linearVelocity += j * getInverseMass();
    }
    float getInverseMass() const { return isStatic || mass <= 0.0f ? 0.0f : 1.0f / mass; }
    void applyForce(const Vec3 &f) {
        if (isStatic) return;
        if (f.x != 0.0f || f.y != 0.0f || f.z != 0.0f) wakeUp();
        force += f;
    }
    void clearForces() { force = Vec3::zero(); }
    Quaternion getRotation() const { return rotation; }
    Vec3 getAngularVelocity() const { return angularVelocity; }
    void setAngularVelocity(const Vec3 &v) {
        wakeUp();
        angularVelocity = v;
    }
    Mat3 getInverseInertiaWorld() const {
        const Mat3 r = rotation.toMat3();
        return r * inverseInertiaLocal * transpose(r);
    }
    void applyImpulse(const Vec3 &impulse, const Vec3 &offset) {
        if (isStatic) return;
        if (impulse.x != 0.0f || impulse.y != 0.0f || impulse.z != 0.0f) wakeUp();
        linearVelocity += impulse * getInverseMass();
        angularVelocity += getInverseInertiaWorld() * Math3d::cross(offset, impulse);
    }

    static bool createSphere(float radius, Vec3 position, float density, bool isStatic, float restitution,
                             float friction, RigidBody &body, std::string &errorMessage) {
        const float p[3] = {position.x, position.y, position.z};
        pe_body_record r{};
        return finishCreate(pe_body_make_sphere(radius, p, density, isStatic, restitution, friction, &r), r, body,
                            errorMessage);
    }
    static bool createBox(float width, float height, float depth, Vec3 position, float density, bool isStatic,
                          float restitution, float friction, RigidBody &body, std::string &errorMessage) {
        const float p[3] = {position.x, position.y, position.z};
        pe_body_record r{};
        return finishCreate(
            pe_body_make_box(width, height, depth, p, density, isStatic, restitution, friction, &r), r, body,
            errorMessage);
    }

  private:
    friend class PhysicsWorld;
    friend class SequentialImpulseSolver;

    static bool finishCreate(pe_status s, const pe_body_record &r, RigidBody &body, std::string &errorMessage) {
        errorMessage.clear();
        if (s == PE_ERR_CREATE_FAILED) {
            errorMessage = pe_last_error();
            return false;
        }
        throwIf(s);
        body.fromRecord(r);
        return true;
    }
    pe_body_record toRecord() const {
        pe_body_record r{};
        const float pv[3] = {position.x, position.y, position.z};
        const float q[4] = {rotation.x, rotation.y, rotation.z, rotation.w};
        const float l[3] = {linearVelocity.x, linearVelocity.y, linearVelocity.z};
        const float a[3] = {angularVelocity.x, angularVelocity.y, angularVelocity.z};
        const float f[3] = {force.x, force.y, force.z};
        for (int k = 0; k < 3; ++k) {
            r.state.position[k] = pv[k];
            r.state.linear_velocity[k] = l[k];
            r.state.angular_velocity[k] = a[k];
            r.state.force[k] = f[k];
        }
        for (int k = 0; k < 4; ++k) r.state.rotation[k] = q[k];
        r.state.mass = mass;
        r.state.restitution = restitution;
        r.state.friction = friction;
        r.state.is_static = isStatic ? 1 : 0;
        // the factories set a diagonal local inverse inertia
        r.inv_inertia[0] = inverseInertiaLocal.m00;
        r.inv_inertia[1] = inverseInertiaLocal.m11;
        r.inv_inertia[2] = inverseInertiaLocal.m22;
        r.sleeping = sleeping ? 1 : 0;
        r.wake_requested = wakeRequested ? 1 : 0;
        return r;
    }
    void fromRecord(const pe_body_record &r) {
        position = {r.state.position[0], r.state.position[1], r.state.position[2]};
        rotation = {r.state.rotation[0], r.state.rotation[1], r.state.rotation[2], r.state.rotation[3]};
        linearVelocity = {r.state.linear_velocity[0], r.state.linear_velocity[1], r.state.linear_velocity[2]};
        angularVelocity = {r.state.angular_velocity[0], r.state.angular_velocity[1], r.state.angular_velocity[2]};
        force = {r.state.force[0], r.state.force[1], r.state.force[2]};
        mass = r.state.mass;
        restitution = r.state.restitution;
        friction = r.state.friction;
        isStatic = r.state.is_static != 0;
        inverseInertiaLocal = Mat3{};
        inverseInertiaLocal.m00 = r.inv_inertia[0];
        inverseInertiaLocal.m11 = r.inv_inertia[1];
        inverseInertiaLocal.m22 = r.inv_inertia[2];
        sleeping = r.sleeping != 0;
        wakeRequested = r.wake_requested != 0;
    }
    bool sameState(const RigidBody &o) const {
        const pe_body_record x = toRecord(), y = o.toRecord();
        for (int k = 0; k < 3; ++k)
            if (x.state.position[k] != y.state.position[k] || x.state.linear_velocity[k] != y.state.linear_velocity[k] ||
                x.state.angular_velocity[k] != y.state.angular_velocity[k] || x.state.force[k] != y.state.force[k] ||
                x.inv_inertia[k] != y.inv_inertia[k])
                return false;
        for (int k = 0; k < 4; ++k)
            if (x.state.rotation[k] != y.state.rotation[k]) return false;
        return x.state.mass == y.state.mass && x.state.restitution == y.state.restitution &&
               x.state.friction == y.state.friction && x.state.is_static == y.state.is_static &&
               x.sleeping == y.sleeping && x.wake_requested == y.wake_requested;
    }
    void integrate(int stage, const float *g, float dt) {
        pe_body_record r = toRecord();
        throwIf(pe_body_integrate(&r, stage, g, dt));
        fromRecord(r);
    }

    bool sleeping = false;
    bool wakeRequested = true;
    Vec3 position{};
    Vec3 linearVelocity{};
    Quaternion rotation = Quaternion::identity();
    Vec3 angularVelocity{};
    Vec3 force{};
    Mat3 inverseInertiaLocal{};
};

namespace detail {
inline int &defaultDevice() {
    static int device = 0;
    return device;
}
inline pe_contact_manifold toNative(const ContactManifold &c) {
    pe_contact_manifold r{};
    r.body_a_index = c.bodyA.index;
    r.body_a_generation = c.bodyA.generation;
    r.body_b_index = c.bodyB.index;
    r.body_b_generation = c.bodyB.generation;
    r.normal[0] = c.normal.x, r.normal[1] = c.normal.y, r.normal[2] = c.normal.z;
    r.point_count = c.pointCount;
    r.friction = c.friction;
    r.restitution = c.restitution;
    for (int k = 0; k < 4; ++k) {
        const ContactPoint &p = c.points[k];
        r.anchor_a[k][0] = p.localAnchorA.x, r.anchor_a[k][1] = p.localAnchorA.y, r.anchor_a[k][2] = p.localAnchorA.z;
        r.anchor_b[k][0] = p.localAnchorB.x, r.anchor_b[k][1] = p.localAnchorB.y, r.anchor_b[k][2] = p.localAnchorB.z;
        r.penetration[k] = p.penetration;
        r.normal_impulse[k] = p.normalImpulse;
        r.tangent_impulse1[k] = p.tangentImpulse1;
        r.tangent_impulse2[k] = p.tangentImpulse2;
        r.feature[k] = p.feature;
    }
    return r;
}
inline void fromNative(const pe_contact_manifold &r, ContactManifold &c, bool handles = true) {
    if (handles) {
        c.bodyA = {r.body_a_index, r.body_a_generation};
        c.bodyB = {r.body_b_index, r.body_b_generation};
    }
    c.normal = {r.normal[0], r.normal[1], r.normal[2]};
    c.pointCount = r.point_count;
    c.friction = r.friction;
    c.restitution = r.restitution;
    for (int k = 0; k < 4; ++k) {
        ContactPoint &p = c.points[k];
        p.localAnchorA = {r.anchor_a[k][0], r.anchor_a[k][1], r.anchor_a[k][2]};
        p.localAnchorB = {r.anchor_b[k][0], r.anchor_b[k][1], r.anchor_b[k][2]};
        p.penetration = r.penetration[k];
        p.normalImpulse = r.normal_impulse[k];
        p.tangentImpulse1 = r.tangent_impulse1[k];
        p.tangentImpulse2 = r.tangent_impulse2[k];
        p.feature = r.feature[k];
    }
}
inline int shapeOf(const Collider &c, float dims[3]) {
    if (const Sphere *s = std::get_if<Sphere>(&c.shape)) {
        dims[0] = s->radius, dims[1] = dims[2] = 0.0f;
        return PE_SHAPE_SPHERE;
    }
    const Box &b = std::get<Box>(c.shape);
    dims[0] = b.halfExtents.x, dims[1] = b.halfExtents.y, dims[2] = b.halfExtents.z;
    return PE_SHAPE_BOX;
}
} // namespace detail

// ---------------------------------------------------------- PhysicsWorld ---
class PhysicsWorld {
  public:
    static constexpr float minBodySize = BodyLimits::minSize;
    static constexpr float maxBodySize = BodyLimits::maxSize;
    static constexpr float minDensity = BodyLimits::minDensity;
    static constexpr float maxDensity = BodyLimits::maxDensity;

    Vec3 gravity{0.0f, -9.81f, 0.0f};
    BroadPhaseAlgorithm broadPhaseAlgorithm = BroadPhaseAlgorithm::SweepAndPrune;

    // The reference's solver: 8 iterations in manifold order (bit-identical results).
    PhysicsWorld() : PhysicsWorld(detail::defaultDevice(), 8, PE_ORDER_MANIFOLD) {}
    PhysicsWorld(int device, int solverIterations, int order) {
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
        o.commit();
        throwIf(pe_world_clone(o.w_, &w_));
    }
    PhysicsWorld &operator=(const PhysicsWorld &o) {
        if (this == &o) return *this;
        o.commit();
        pe_world *c = nullptr;
        throwIf(pe_world_clone(o.w_, &c));
        reset();
        w_ = c;
        copySettings(o);
        return *this;
    }
    PhysicsWorld(PhysicsWorld &&o) noexcept { take(o); }
    PhysicsWorld &operator=(PhysicsWorld &&o) noexcept {
        if (this != &o) {
            reset();
            take(o);
        }
        return *this;
    }

    RigidBodyHandle addBody(const RigidBody &body) {
        commit();
        const pe_body_record r = body.toRecord();
        pe_handle h{};
        throwIf(pe_world_add_body(w_, &r, &h));
        changed();
        return {h.index, h.generation};
    }
    void removeBody(RigidBodyHandle h) {
        commit();
        throwIf(pe_world_remove_body(w_, pe_handle{h.index, h.generation}));
        changed();
    }
    bool createSphere(float radius, Vec3 position, float density, bool isStatic, float restitution, float friction,
                      RigidBodyHandle &body, ColliderHandle &collider, std::string &errorMessage) {
        commit();
        errorMessage.clear();
        const float p[3] = {position.x, position.y, position.z};
        pe_handle b{}, c{};
        return finishCreate(pe_world_create_sphere(w_, radius, p, density, isStatic, restitution, friction, &b, &c),
                            b, c, body, collider, errorMessage);
    }
    bool createBox(float width, float height, float depth, Vec3 position, float density, bool isStatic,
                   float restitution, float friction, RigidBodyHandle &body, ColliderHandle &collider,
                   std::string &errorMessage) {
        commit();
        errorMessage.clear();
        const float p[3] = {position.x, position.y, position.z};
        pe_handle b{}, c{};
        return finishCreate(
            pe_world_create_box(w_, width, height, depth, p, density, isStatic, restitution, friction, &b, &c), b, c,
            body, collider, errorMessage);
    }

    // nullptr for a stale handle.  The pointee is a host copy owned by this
    // world: edits made through it are written back at the world's next call,
    // and it is brought up to date after every step, solve or wake-up.
    RigidBody *getBody(RigidBodyHandle h) { return fetchBody(h); }
    const RigidBody *getBody(RigidBodyHandle h) const { return fetchBody(h); }

    // An empty handle for a stale body (physics_world.cpp:276-281).
    ColliderHandle addCollider(const Collider &c) {
        commit();
        float d[3];
        const int shape = detail::shapeOf(c, d);
        const Vec3 &lp = c.localTransform.position;
        const Quaternion &lq = c.localTransform.orientation;
        const float p[3] = {lp.x, lp.y, lp.z}, q[4] = {lq.x, lq.y, lq.z, lq.w};
        pe_handle out{};
        const pe_status s = pe_world_add_collider(w_, pe_handle{c.body.index, c.body.generation}, shape, d, p, q, &out);
        if (s == PE_ERR_STALE_HANDLE) return {};
        throwIf(s);
        changed();
        return {out.index, out.generation};
    }
    void removeCollider(ColliderHandle h) {
        commit();
        throwIf(pe_world_remove_collider(w_, pe_handle{h.index, h.generation}));
        changed();
    }
    Collider *getCollider(ColliderHandle h) { return fetchCollider(h); }
    const Collider *getCollider(ColliderHandle h) const { return fetchCollider(h); }

    const std::vector<ContactManifold> &contacts() const {
        commit();
        if (!contactsValid_) {
            uint32_t n = 0;
            const pe_status s = pe_world_get_contacts(w_, nullptr, 0, &n);
            if (s != PE_OK && s != PE_ERR_CAPACITY) throwIf(s);
            std::vector<pe_contact_manifold> raw(n);
            if (n) throwIf(pe_world_get_contacts(w_, raw.data(), n, &n));
            contacts_.assign(n, ContactManifold{});
            for (uint32_t m = 0; m < n; ++m) detail::fromNative(raw[m], contacts_[m]);
            contactsValid_ = true;
        }
        return contacts_;
    }

    void setSleepingEnabled(bool enabled) {
        commit();
        throwIf(pe_world_set_sleeping_enabled(w_, enabled));
        changed();
    }
    bool isSleepingEnabled() const {
        int v = 0;
        throwIf(pe_world_get_sleeping_enabled(w_, &v));
        return v != 0;
    }
    // Worker counts keep the reference's validation (zero throws
    // std::invalid_argument); the device does not use host threads.
    void setNarrowPhaseWorkerCount(std::size_t n) { setWorkers(n, solverWorkers_, broadWorkers_, &npWorkers_); }
    std::size_t getNarrowPhaseWorkerCount() const { return npWorkers_; }
    void setSolverWorkerCount(std::size_t n) { setWorkers(npWorkers_, n, broadWorkers_, &solverWorkers_); }
    std::size_t getSolverWorkerCount() const { return solverWorkers_; }
    void setBroadPhaseWorkerCount(std::size_t n) { setWorkers(npWorkers_, solverWorkers_, n, &broadWorkers_); }
    std::size_t getBroadPhaseWorkerCount() const { return broadWorkers_; }

    void step(float dt) {
        commit();
        throwIf(pe_world_set_gravity(w_, gravity.x, gravity.y, gravity.z));
        throwIf(pe_world_set_broadphase(w_, broadPhaseAlgorithm == BroadPhaseAlgorithm::UniformGrid ? PE_BROADPHASE_GRID
                                            : broadPhaseAlgorithm == BroadPhaseAlgorithm::DynamicTree ? PE_BROADPHASE_TREE
                                                                                                       : PE_BROADPHASE_SAP));
        throwIf(pe_world_step(w_, dt));
        changed();
        statsFromStep_ = true;
    }

    const StepStats &lastStepStats() const {
        commit();
        if (!statsValid_) {
            pe_step_stats s{};
            throwIf(pe_world_get_step_stats(w_, &s));
            StepStats &t = stats_;
            const SolverStats keep = t.solverDetails;
            t = StepStats{};
            t.totalMs = s.total_ms;
            t.integrateVelocityMs = s.integrate_ms;
            t.broadPhaseMs = s.broadphase_ms;
            t.narrowPhaseMs = s.narrowphase_ms;
            t.solverMs = s.solver_ms;
            t.integratePoseMs = s.pose_ms;
            BroadPhaseStats &b = t.broadPhaseDetails;
            b.sweepMs = s.broadphase_ms;
            b.xWindowComparisons = s.x_window_comparisons;
            b.aabbPairs = s.aabb_pairs;
            b.gridComparisons = s.grid_comparisons;
            b.gridEntries = s.grid_entries;
            b.gridOverflowAabbs = s.grid_overflow_aabbs;
            b.gridCellSize = s.grid_cell_size;
            NarrowPhaseStats &n = t.narrowPhaseDetails;
            n.sphereSphereCandidates = s.np_candidates[0];
            n.sphereBoxCandidates = s.np_candidates[1];
            n.boxBoxCandidates = s.np_candidates[2];
            n.sphereSphereContacts = s.np_contacts[0];
            n.sphereBoxContacts = s.np_contacts[1];
            n.boxBoxContacts = s.np_contacts[2];
            SolverStats &v = t.solverDetails;
            v.velocityIterationsMs = s.solver_ms;
            v.preparedPoints = s.prepared_points;
            v.warmStartComparisons = s.warm_start_comparisons;
            v.warmStartMatches = s.warm_start_matches;
            v.velocityPointVisits = s.velocity_point_visits;
            if (statsFromStep_) {
                t.possiblePairs = s.possible_pairs;
                t.candidatePairs = s.candidate_pairs;
                t.contactCount = s.contact_count;
                t.solvedContactCount = s.solved_contact_count;
                t.awakeBodyCount = s.awake_body_count;
                t.sleepingBodyCount = s.sleeping_body_count;
                islandStats(contacts(), v);
            } else {
                // after SequentialImpulseSolver::solve only the solver's
                // details change (the step counters are the last step's)
                t.possiblePairs = keptStep_.possiblePairs;
                t.candidatePairs = keptStep_.candidatePairs;
                t.contactCount = keptStep_.contactCount;
                t.solvedContactCount = s.solved_contact_count;
                t.awakeBodyCount = keptStep_.awakeBodyCount;
                t.sleepingBodyCount = keptStep_.sleepingBodyCount;
                v.islandCount = keep.islandCount;
                v.largestIslandContacts = keep.largestIslandContacts;
                v.largestIslandPoints = keep.largestIslandPoints;
            }
            statsValid_ = true;
        }
        return stats_;
    }
    // The device counters of the last step or solve (GPU detail: colours,
    // EPA failures, device times per stage, graph replay).
    pe_step_stats lastDeviceStats() const {
        pe_step_stats s{};
        throwIf(pe_world_get_step_stats(w_, &s));
        return s;
    }

    pe_world *native() const {
        commit();
        return w_;
    }
    // Device used by default-constructed worlds and the BroadPhase /
    // NarrowPhase statics.
    static void setDevice(int device) { detail::defaultDevice() = device; }

  private:
    friend class SequentialImpulseSolver;
    struct BodyEntry {
        RigidBody body, snapshot;
        RigidBodyHandle handle;
    };
    struct ColliderEntry {
        Collider collider, snapshot;
        ColliderHandle handle;
    };

    RigidBody *fetchBody(RigidBodyHandle h) const {
        commit();
        pe_body_record r{};
        const pe_status s = pe_world_get_body_record(w_, pe_handle{h.index, h.generation}, &r);
        if (s == PE_ERR_STALE_HANDLE) return nullptr;
        throwIf(s);
        std::unique_ptr<BodyEntry> &e = bodies_[h.index];
        if (!e) e = std::make_unique<BodyEntry>();
        e->body.fromRecord(r);
        e->snapshot = e->body;
        e->handle = h;
        return &e->body;
    }
    Collider *fetchCollider(ColliderHandle h) const {
        commit();
        pe_handle body{};
        int shape = 0;
        float d[3], p[3], q[4];
        const pe_status s = pe_world_get_collider(w_, pe_handle{h.index, h.generation}, &body, &shape, d, p, q);
        if (s == PE_ERR_STALE_HANDLE) return nullptr;
        throwIf(s);
        std::unique_ptr<ColliderEntry> &e = colliders_[h.index];
        if (!e) e = std::make_unique<ColliderEntry>();
        Collider &c = e->collider;
        c.body = {body.index, body.generation};
        c.localTransform = Transform({p[0], p[1], p[2]}, Quaternion{q[0], q[1], q[2], q[3]});
        if (shape == PE_SHAPE_SPHERE) c.shape = Sphere{d[0]};
        else c.shape = Box{{d[0], d[1], d[2]}};
        c.bounds = Aabb{};
        e->snapshot = c;
        e->handle = h;
        return &c;
    }
    // Writes back what callers changed through getBody / getCollider pointers
    // (every copy handed out so far is watched).
    void commit() const {
        bool any = false;
        for (auto &kv : bodies_) {
            BodyEntry *e = kv.second.get();
            const RigidBody &b = e->body;
            const RigidBody s = e->snapshot;
            const pe_handle h{e->handle.index, e->handle.generation};
            if (b.sameState(s)) continue;
            e->snapshot = b;
            const pe_body_record r = b.toRecord();
            const pe_status st = pe_world_set_body(w_, h, &r.state);
            if (st == PE_ERR_STALE_HANDLE) continue;  // a removed body's copy
            throwIf(st);
            if ((b.wakeRequested && !s.wakeRequested) || (!b.sleeping && s.sleeping)) throwIf(pe_world_body_wake_up(w_, h));
            any = true;
        }
        for (auto &kv : colliders_) {
            ColliderEntry *e = kv.second.get();
            float d[3], sd[3];
            const int shape = detail::shapeOf(e->collider, d), sshape = detail::shapeOf(e->snapshot, sd);
            const Collider &c = e->collider;
            const Collider s = e->snapshot;
            const Vec3 &lp = c.localTransform.position;
            const Quaternion &lq = c.localTransform.orientation;
            const float p[3] = {lp.x, lp.y, lp.z}, q[4] = {lq.x, lq.y, lq.z, lq.w};
            const Vec3 &sp = s.localTransform.position;
            const Quaternion &sq = s.localTransform.orientation;
            const bool same = shape == sshape && d[0] == sd[0] && d[1] == sd[1] && d[2] == sd[2] && c.body == s.body &&
                              lp.x == sp.x && lp.y == sp.y && lp.z == sp.z && lq.x == sq.x && lq.y == sq.y &&
                              lq.z == sq.z && lq.w == sq.w;
            if (same) continue;
            e->snapshot = c;
            const pe_status st = pe_world_set_collider(w_, pe_handle{e->handle.index, e->handle.generation},
                                                       pe_handle{c.body.index, c.body.generation}, shape, d, p, q);
            if (st == PE_ERR_STALE_HANDLE) continue;
            throwIf(st);
            any = true;
        }
        if (any) refreshBodies();  // geometry edits wake bodies
    }
    // After anything that changes body state on the device (a step, a solve,
    // wake-ups), the host copies handed out so far show the new state.
    void refreshBodies() const {
        for (auto &kv : bodies_) {
            BodyEntry *e = kv.second.get();
            pe_body_record r{};
            if (pe_world_get_body_record(w_, pe_handle{e->handle.index, e->handle.generation}, &r) != PE_OK) continue;
            e->body.fromRecord(r);
            e->snapshot = e->body;
        }
    }
    void changed() const {
        contactsValid_ = false;
        statsValid_ = false;
        refreshBodies();
    }
    // SolverStats island counters (sequential_impulse_solver.cpp:366-442): the
    // reference fills them when its island-parallel solve runs (more than one
    // solver worker and at least 4,096 contacts).
    void islandStats(const std::vector<ContactManifold> &cs, SolverStats &v) const {
        v.islandCount = v.largestIslandContacts = v.largestIslandPoints = 0;
        if (solverWorkers_ <= 1 || cs.size() < 4096) return;
        std::unordered_map<uint32_t, uint32_t> parent;
        std::unordered_map<uint32_t, bool> isStatic;
        auto staticOf = [&](RigidBodyHandle h) {
            auto it = isStatic.find(h.index);
            if (it != isStatic.end()) return it->second;
            pe_body_record r{};
            const bool st = pe_world_get_body_record(w_, pe_handle{h.index, h.generation}, &r) != PE_OK ||
                            r.state.is_static != 0;
            isStatic[h.index] = st;
            return st;
        };
        auto root = [&](uint32_t i) {
            if (!parent.count(i)) parent[i] = i;
            while (parent[i] != i) i = parent[i] = parent[parent[i]];
            return i;
        };
        for (const ContactManifold &m : cs) {
            if (staticOf(m.bodyA) || staticOf(m.bodyB)) continue;
            const uint32_t a = root(m.bodyA.index), b = root(m.bodyB.index);
            if (a != b) parent[std::max(a, b)] = std::min(a, b);
        }
        std::unordered_map<uint32_t, std::pair<std::size_t, std::size_t>> count;
        for (const ContactManifold &m : cs) {
            const uint32_t r = root(staticOf(m.bodyA) ? m.bodyB.index : m.bodyA.index);
            count[r].first += 1;
            count[r].second += m.pointCount;
        }
        v.islandCount = count.size();
        for (const auto &kv : count) {
            v.largestIslandContacts = std::max(v.largestIslandContacts, kv.second.first);
            v.largestIslandPoints = std::max(v.largestIslandPoints, kv.second.second);
        }
    }
    bool finishCreate(pe_status s, pe_handle b, pe_handle c, RigidBodyHandle &body, ColliderHandle &collider,
                      std::string &errorMessage) {
        if (s == PE_ERR_CREATE_FAILED) {
            errorMessage = pe_last_error();
            return false;
        }
        throwIf(s);
        changed();
        body = {b.index, b.generation};
        collider = {c.index, c.generation};
        return true;
    }
    void setWorkers(std::size_t np, std::size_t solver, std::size_t bp, std::size_t *which) {
        throwIf(pe_world_set_worker_counts(w_, np, solver, bp));
        *which = which == &npWorkers_ ? np : which == &solverWorkers_ ? solver : bp;
    }
    void copySettings(const PhysicsWorld &o) {
        gravity = o.gravity;
        broadPhaseAlgorithm = o.broadPhaseAlgorithm;
        npWorkers_ = o.npWorkers_;
        solverWorkers_ = o.solverWorkers_;
        broadWorkers_ = o.broadWorkers_;
    }
    void reset() {
        if (w_) pe_world_destroy(w_);
        w_ = nullptr;
        bodies_.clear();
        colliders_.clear();
        contactsValid_ = false;
        statsValid_ = false;
    }
    void take(PhysicsWorld &o) {
        w_ = o.w_;
        o.w_ = nullptr;
        copySettings(o);
        bodies_ = std::move(o.bodies_);
        colliders_ = std::move(o.colliders_);
        contacts_ = std::move(o.contacts_);
        contactsValid_ = o.contactsValid_;
        stats_ = o.stats_;
        statsValid_ = o.statsValid_;
        statsFromStep_ = o.statsFromStep_;
        keptStep_ = o.keptStep_;
        o.bodies_.clear();
        o.colliders_.clear();
    }

    pe_world *w_ = nullptr;
    std::size_t npWorkers_ = 1, solverWorkers_ = 1, broadWorkers_ = 1;
    mutable std::unordered_map<uint32_t, std::unique_ptr<BodyEntry>> bodies_;
    mutable std::unordered_map<uint32_t, std::unique_ptr<ColliderEntry>> colliders_;
    mutable std::vector<ContactManifold> contacts_;
    mutable bool contactsValid_ = false;
    mutable StepStats stats_{};
    mutable bool statsValid_ = false;
    bool statsFromStep_ = true;
    StepStats keptStep_{};
};


// ------------------------------------------------------------ the statics ---
class SequentialImpulseSolver {
  public:
    // Solves `contacts` against the world's bodies (the world's solver order
    // and iterations), writing impulses back into the vector.
    static void solve(std::vector<ContactManifold> &contacts, PhysicsWorld &world, float dt) {
        world.commit();
        std::vector<pe_contact_manifold> raw(contacts.size());
        for (std::size_t m = 0; m < contacts.size(); ++m) raw[m] = detail::toNative(contacts[m]);
        if (!world.statsValid_) world.lastStepStats();
        world.keptStep_ = world.stats_;
        throwIf(pe_world_solve(world.w_, raw.data(), (uint32_t)raw.size(), dt));
        for (std::size_t m = 0; m < contacts.size(); ++m) detail::fromNative(raw[m], contacts[m], false);
        world.changed();
        world.statsFromStep_ = false;
        world.lastStepStats();
        world.islandStats(contacts, world.stats_.solverDetails);
    }
};

class BroadPhase {
  public:
    // Touching boxes pair; bounds finite with min <= max; pairs in
    // lexicographic order with first < second; stats overwritten.
    static std::vector<BroadPhasePair> findCandidatePairs(const std::vector<Aabb> &bounds,
                                                          BroadPhaseStats *stats = nullptr,
                                                          BroadPhaseAlgorithm algorithm =
                                                              BroadPhaseAlgorithm::SweepAndPrune) {
        if (algorithm == BroadPhaseAlgorithm::DynamicTree)
            throw std::invalid_argument("DynamicTree broadphase requires a persistent DynamicAabbTree");
        const uint32_t n = (uint32_t)bounds.size();
        std::vector<float> mn(3 * (size_t)n), mx(3 * (size_t)n);
        for (uint32_t i = 0; i < n; ++i) {
            mn[3 * i] = bounds[i].min.x, mn[3 * i + 1] = bounds[i].min.y, mn[3 * i + 2] = bounds[i].min.z;
            mx[3 * i] = bounds[i].max.x, mx[3 * i + 1] = bounds[i].max.y, mx[3 * i + 2] = bounds[i].max.z;
        }
        const int algo = algorithm == BroadPhaseAlgorithm::UniformGrid ? PE_BROADPHASE_GRID : PE_BROADPHASE_SAP;
        uint64_t count = 0;
        pe_step_stats st{};
        pe_status s = pe_broadphase_find_pairs(detail::defaultDevice(), mn.data(), mx.data(), n, algo, 0.0, nullptr,
                                               0, &count, &st);
        if (s != PE_OK && s != PE_ERR_CAPACITY) throwIf(s);
        std::vector<uint32_t> raw(2 * count);
        if (count)
            throwIf(pe_broadphase_find_pairs(detail::defaultDevice(), mn.data(), mx.data(), n, algo, 0.0, raw.data(),
                                             count, &count, &st));
        std::vector<BroadPhasePair> pairs(count);
        for (uint64_t k = 0; k < count; ++k) pairs[k] = {raw[2 * k], raw[2 * k + 1]};
        if (stats) {
            *stats = BroadPhaseStats{};
            stats->xWindowComparisons = st.x_window_comparisons;
            stats->aabbPairs = st.aabb_pairs;
            stats->gridComparisons = st.grid_comparisons;
            stats->gridEntries = st.grid_entries;
            stats->gridOverflowAabbs = st.grid_overflow_aabbs;
            stats->gridCellSize = st.grid_cell_size;
        }
        return pairs;
    }
};

class NarrowPhase {
  public:
    static bool intersectSphereSphere(const Sphere &a, const Transform &ta, const Sphere &b, const Transform &tb,
                                      ContactManifold &m) {
        const float da[3] = {a.radius, 0, 0}, db[3] = {b.radius, 0, 0};
        return run(PE_SHAPE_SPHERE, da, ta, PE_SHAPE_SPHERE, db, tb, m);
    }
    static bool intersectSphereBox(const Sphere &s, const Transform &ts, const Box &b, const Transform &tb,
                                   ContactManifold &m) {
        const float ds[3] = {s.radius, 0, 0}, db[3] = {b.halfExtents.x, b.halfExtents.y, b.halfExtents.z};
        return run(PE_SHAPE_SPHERE, ds, ts, PE_SHAPE_BOX, db, tb, m);
    }
    static bool intersectBoxBox(const Box &a, const Transform &ta, const Box &b, const Transform &tb,
                                ContactManifold &m) {
        const float da[3] = {a.halfExtents.x, a.halfExtents.y, a.halfExtents.z};
        const float db[3] = {b.halfExtents.x, b.halfExtents.y, b.halfExtents.z};
        return run(PE_SHAPE_BOX, da, ta, PE_SHAPE_BOX, db, tb, m);
    }
    // Colliders at the given world transforms (their localTransform is not
    // applied, as in the reference); the manifold is reset and takes the
    // colliders' bodies.
    static bool generateContact(const Collider &a, const Transform &ta, const Collider &b, const Transform &tb,
                                ContactManifold &m) {
        m = ContactManifold{};
        m.bodyA = a.body;
        m.bodyB = b.body;
        float da[3], db[3];
        const int sa = detail::shapeOf(a, da), sb = detail::shapeOf(b, db);
        return run(sa, da, ta, sb, db, tb, m);
    }

  private:
    static bool run(int sa, const float *da, const Transform &ta, int sb, const float *db, const Transform &tb,
                    ContactManifold &m) {
        const float pa[3] = {ta.position.x, ta.position.y, ta.position.z};
        const float qa[4] = {ta.orientation.x, ta.orientation.y, ta.orientation.z, ta.orientation.w};
        const float pb[3] = {tb.position.x, tb.position.y, tb.position.z};
        const float qb[4] = {tb.orientation.x, tb.orientation.y, tb.orientation.z, tb.orientation.w};
        pe_contact_manifold out{};
        int hit = 0;
        throwIf(pe_generate_contact(detail::defaultDevice(), sa, da, pa, qa, sb, db, pb, qb, &out, &hit));
        if (hit) detail::fromNative(out, m, false);
        return hit != 0;
    }
};

} // namespace phys_gb300
