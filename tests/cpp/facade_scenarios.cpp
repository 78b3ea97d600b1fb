// Scenarios of the reference's solver and sleeping tests
// (tests/solver/sequential_impulse_solver_tests.cpp:293-378,
// tests/world/sleeping_tests.cpp of bkuangs/phys-engine)
// written against the phys_gb300 facade the way a caller of phys::PhysicsWorld
// writes them; links libphys_gb300.so and runs on the GPU.  Exit code 0 = pass.
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <utility>

#include "phys_gb300_world.hpp"

using namespace phys_gb300;

static bool boxLandsOnStaticFloor() {
    PhysicsWorld world;
    world.gravity = {0.0f, -9.81f, 0.0f};
    RigidBodyHandle floorBody, boxBody;
    ColliderHandle floorCollider, boxCollider;
    std::string error;
    if (!world.createBox(18.0f, 1.0f, 8.0f, {0.0f, -0.5f, 0.0f}, 1.0f, true, 0.1f, 0.6f, floorBody, floorCollider,
                         error) ||
        !world.createBox(1.4f, 1.4f, 1.4f, {-1.5f, 3.0f, 0.0f}, 1.0f, false, 0.2f, 0.5f, boxBody, boxCollider,
                         error)) {
        std::fprintf(stderr, "creation failed: %s\n", error.c_str());
        return false;
    }
    for (int step = 0; step < 180; ++step) world.step(1.0f / 60.0f);
    BodyRef body = world.getBody(boxBody);
    auto contacts = world.contacts();
    bool ok = body && body.getPosition().y >= 0.68f && body.getPosition().y <= 0.72f &&
              std::fabs(body.getPosition().x + 1.5f) <= 0.02f && std::fabs(body.getLinearVelocity().x) <= 0.02f &&
              std::fabs(body.getAngularVelocity().z) <= 0.02f && !contacts.empty() && contacts.front().pointCount >= 2;
    if (!ok) std::fprintf(stderr, "box did not land: y=%f contacts=%zu\n", body.getPosition().y, contacts.size());
    return ok;
}

static bool tiltedBoxSettlesFlat(float dt, float angle, Vec3 axis) {
    PhysicsWorld world(0, 8, PE_ORDER_COLOR);
    RigidBodyHandle floorBody, boxBody;
    ColliderHandle floorCollider, boxCollider;
    std::string error;
    if (!world.createBox(18.0f, 1.0f, 8.0f, {0.0f, -0.5f, 0.0f}, 1.0f, true, 0.0f, 0.6f, floorBody, floorCollider,
                         error) ||
        !world.createBox(1.0f, 1.0f, 1.0f, {0.0f, 2.0f, 0.0f}, 1.0f, false, 0.0f, 0.55f, boxBody, boxCollider, error))
        return false;
    BodyRef body = world.getBody(boxBody);
    float s = 2.0f * std::tan(angle * 0.5f);
    body.setAngularVelocity({axis.x * s, axis.y * s, axis.z * s});
    body.integrateRotation(1.0f);
    body.setAngularVelocity({});
    for (int step = 0; step < 600; ++step) world.step(dt);
    body = world.getBody(boxBody);
    Quaternion q = body.getRotation();
    // y of the rotated unit axes: the box is flat when one of them is ~vertical
    float ax = std::fabs(2.0f * (q.x * q.y + q.w * q.z));
    float ay = std::fabs(1.0f - 2.0f * (q.x * q.x + q.z * q.z));
    float az = std::fabs(2.0f * (q.y * q.z - q.w * q.x));
    float alignment = std::fmax(ax, std::fmax(ay, az));
    Vec3 v = body.getLinearVelocity(), w = body.getAngularVelocity();
    bool ok = alignment >= 0.995f && std::fabs(body.getPosition().y - 0.5f) <= 0.03f &&
              std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z) <= 0.08f &&
              std::sqrt(w.x * w.x + w.y * w.y + w.z * w.z) <= 0.1f;
    if (!ok) std::fprintf(stderr, "tilted box: alignment=%f y=%f\n", alignment, body.getPosition().y);
    return ok;
}

static bool invalidInputs() {
    PhysicsWorld world;
    RigidBodyHandle b;
    ColliderHandle c;
    std::string error;
    if (world.createSphere(0.001f, {}, 1.0f, false, 0, 0, b, c, error) || error != "Sphere is too small") return false;
    if (world.createBox(1, 1, 1, {}, 30.0f, false, 0, 0, b, c, error) || error != "Density is out of range") return false;
    try {
        world.setSolverWorkerCount(0);
        return false;
    } catch (const std::invalid_argument &) {
    }
    if (world.getBody(RigidBodyHandle{7, 3})) return false;  // stale handle -> "nullptr"
    // the tree selector steps like the others (same candidate pairs)
    world.broadPhaseAlgorithm = BroadPhaseAlgorithm::DynamicTree;
    if (!world.createSphere(0.5f, {0, 0, 0}, 1.0f, false, 0, 0, b, c, error) ||
        !world.createSphere(0.5f, {0.9f, 0, 0}, 1.0f, false, 0, 0, b, c, error))
        return false;
    world.step(1.0f / 60.0f);
    return world.contacts().size() == 1 && world.lastStepStats().candidate_pairs == 1;
}

// Opt-in sleeping of a settled stack, after tests/world/sleeping_tests.cpp:72-110
// and :172-200 of the reference.
static bool settledStackSleepsAndWakes() {
    const float dt = 1.0f / 120.0f;
    PhysicsWorld world;
    RigidBodyHandle floorBody, lower, upper, other;
    ColliderHandle c;
    std::string error;
    if (!world.createBox(10, 1, 10, {0, -0.5f, 0}, 1, true, 0, 0.6f, floorBody, c, error) ||
        !world.createBox(1, 1, 1, {0, 0.5f, 0}, 1, false, 0, 0.6f, lower, c, error) ||
        !world.createBox(1, 1, 1, {0, 1.52f, 0}, 1, false, 0, 0.6f, upper, c, error) ||
        !world.createBox(1, 1, 1, {3, 0.5f, 0}, 1, false, 0, 0.6f, other, c, error))
        return false;
    for (int i = 0; i < 360; ++i) world.step(dt);
    if (world.isSleepingEnabled() || world.lastStepStats().awake_body_count != 3 ||
        world.lastStepStats().solved_contact_count != 3)
        return false;
    world.setSleepingEnabled(true);
    for (int i = 0; i < 120; ++i) world.step(dt);
    StepStats st = world.lastStepStats();
    if (!world.isSleepingEnabled() || st.sleeping_body_count != 3 || st.awake_body_count != 0 ||
        st.solved_contact_count != 0 || world.contacts().size() != 3) {
        std::fprintf(stderr, "stack did not sleep: %llu asleep\n", (unsigned long long)st.sleeping_body_count);
        return false;
    }
    Vec3 p0 = world.getBody(upper).getPosition();
    world.getBody(upper).applyForce({});
    world.getBody(upper).applyLinearImpulse({});
    for (int i = 0; i < 60; ++i) world.step(dt);
    BodyRef u = world.getBody(upper);
    Vec3 p1 = u.getPosition();
    if (!u.isSleeping() || p0.x != p1.x || p0.y != p1.y || p0.z != p1.z) return false;
    for (const ContactManifold &m : world.contacts())
        if (m.pointCount != 4) return false;
    world.getBody(upper).applyForce({0.1f, 0, 0});
    if (world.getBody(upper).isSleeping()) return false;
    world.step(dt);
    if (world.getBody(lower).isSleeping() || world.getBody(upper).isSleeping() || !world.getBody(other).isSleeping() ||
        world.lastStepStats().solved_contact_count != 2)
        return false;
    // copies and moves own independent state (sleeping_tests.cpp:330-343)
    for (int i = 0; i < 120; ++i) world.step(dt);
    PhysicsWorld copied = world;
    PhysicsWorld moved = std::move(copied);
    moved.step(dt);
    if (moved.lastStepStats().sleeping_body_count != 3 || moved.lastStepStats().solved_contact_count != 0)
        return false;
    moved.getBody(upper).wakeUp();
    moved.step(dt);
    if (moved.getBody(lower).isSleeping() || !world.getBody(lower).isSleeping()) return false;
    world.setSleepingEnabled(false);
    if (world.getBody(other).isSleeping()) return false;
    world.step(dt);
    return world.lastStepStats().sleeping_body_count == 0 && world.lastStepStats().solved_contact_count == 3;
}

int main() {
    bool ok = boxLandsOnStaticFloor() && tiltedBoxSettlesFlat(1.0f / 60.0f, 0.6f, {0.0f, 0.0f, 1.0f}) &&
              tiltedBoxSettlesFlat(1.0f / 120.0f, 0.9f, {0.6f, 0.0f, 0.8f}) && invalidInputs() &&
              settledStackSleepsAndWakes();
    std::printf("%s\n", ok ? "facade scenarios ok" : "facade scenarios FAILED");
    return ok ? 0 : 1;
}
