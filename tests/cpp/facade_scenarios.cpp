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
#include <variant>
#include <vector>

#include "phys_gb300_world.hpp"

using namespace phys_gb300;

// Reports the source line of a failed check.
static bool fail(int line) {
    std::fprintf(stderr, "check failed at facade_scenarios.cpp:%d\n", line);
    return false;
}

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
        return fail(29);
    }
    for (int step = 0; step < 180; ++step) world.step(1.0f / 60.0f);
    const RigidBody *body = world.getBody(boxBody);
    const std::vector<ContactManifold> &contacts = world.contacts();
    bool ok = body && body->getPosition().y >= 0.68f && body->getPosition().y <= 0.72f &&
              std::fabs(body->getPosition().x + 1.5f) <= 0.02f && std::fabs(body->getLinearVelocity().x) <= 0.02f &&
              std::fabs(body->getAngularVelocity().z) <= 0.02f && !contacts.empty() && contacts.front().pointCount >= 2;
    if (!ok) std::fprintf(stderr, "box did not land: y=%f contacts=%zu\n", body ? body->getPosition().y : -1.0f,
                          contacts.size());
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
        return fail(50);
    RigidBody *body = world.getBody(boxBody);
    float s = 2.0f * std::tan(angle * 0.5f);
    body->setAngularVelocity({axis.x * s, axis.y * s, axis.z * s});
    body->integrateRotation(1.0f);
    body->setAngularVelocity({});
    for (int step = 0; step < 600; ++step) world.step(dt);
    body = world.getBody(boxBody);
    Quaternion q = body->getRotation();
    // y of the rotated unit axes: the box is flat when one of them is ~vertical
    float ax = std::fabs(2.0f * (q.x * q.y + q.w * q.z));
    float ay = std::fabs(1.0f - 2.0f * (q.x * q.x + q.z * q.z));
    float az = std::fabs(2.0f * (q.y * q.z - q.w * q.x));
    float alignment = std::fmax(ax, std::fmax(ay, az));
    Vec3 v = body->getLinearVelocity(), w = body->getAngularVelocity();
    bool ok = alignment >= 0.995f && std::fabs(body->getPosition().y - 0.5f) <= 0.03f &&
              std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z) <= 0.08f &&
              std::sqrt(w.x * w.x + w.y * w.y + w.z * w.z) <= 0.1f;
    if (!ok) std::fprintf(stderr, "tilted box: alignment=%f y=%f\n", alignment, body->getPosition().y);
    return ok;
}

static bool invalidInputs() {
    PhysicsWorld world;
    RigidBodyHandle b;
    ColliderHandle c;
    std::string error;
    if (world.createSphere(0.001f, {}, 1.0f, false, 0, 0, b, c, error) || error != "Sphere is too small") return fail(77);
    if (world.createBox(1, 1, 1, {}, 30.0f, false, 0, 0, b, c, error) || error != "Density is out of range") return fail(78);
    try {
        world.setSolverWorkerCount(0);
        return fail(81);
    } catch (const std::invalid_argument &) {
    }
    if (world.getBody(RigidBodyHandle{7, 3})) return fail(84);  // stale handle -> "nullptr"
    // the tree selector steps like the others (same candidate pairs)
    world.broadPhaseAlgorithm = BroadPhaseAlgorithm::DynamicTree;
    if (!world.createSphere(0.5f, {0, 0, 0}, 1.0f, false, 0, 0, b, c, error) ||
        !world.createSphere(0.5f, {0.9f, 0, 0}, 1.0f, false, 0, 0, b, c, error))
        return fail(89);
    world.step(1.0f / 60.0f);
    return world.contacts().size() == 1 && world.lastStepStats().candidatePairs == 1;
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
        return fail(106);
    for (int i = 0; i < 360; ++i) world.step(dt);
    if (world.isSleepingEnabled() || world.lastStepStats().awakeBodyCount != 3 ||
        world.lastStepStats().solvedContactCount != 3)
        return fail(110);
    world.setSleepingEnabled(true);
    for (int i = 0; i < 120; ++i) world.step(dt);
    const StepStats &st = world.lastStepStats();
    if (!world.isSleepingEnabled() || st.sleepingBodyCount != 3 || st.awakeBodyCount != 0 ||
        st.solvedContactCount != 0 || world.contacts().size() != 3) {
        std::fprintf(stderr, "stack did not sleep: %llu asleep\n", (unsigned long long)st.sleepingBodyCount);
        return fail(117);
    }
    Vec3 p0 = world.getBody(upper)->getPosition();
    world.getBody(upper)->applyForce({});
    world.getBody(upper)->applyLinearImpulse({});
    for (int i = 0; i < 60; ++i) world.step(dt);
    const RigidBody *u = world.getBody(upper);
    Vec3 p1 = u->getPosition();
    if (!u->isSleeping() || p0.x != p1.x || p0.y != p1.y || p0.z != p1.z) return fail(125);
    for (const ContactManifold &m : world.contacts())
        if (m.pointCount != 4) return fail(127);
    world.getBody(upper)->applyForce({0.1f, 0, 0});
    if (world.getBody(upper)->isSleeping()) return fail(129);
    world.step(dt);
    if (world.getBody(lower)->isSleeping() || world.getBody(upper)->isSleeping() || !world.getBody(other)->isSleeping() ||
        world.lastStepStats().solvedContactCount != 2)
        return fail(133);
    // copies and moves own independent state (sleeping_tests.cpp:330-343)
    for (int i = 0; i < 120; ++i) world.step(dt);
    PhysicsWorld copied = world;
    PhysicsWorld moved = std::move(copied);
    moved.step(dt);
    if (moved.lastStepStats().sleepingBodyCount != 3 || moved.lastStepStats().solvedContactCount != 0)
        return fail(140);
    moved.getBody(upper)->wakeUp();
    moved.step(dt);
    if (moved.getBody(lower)->isSleeping() || !world.getBody(lower)->isSleeping()) return fail(143);
    world.setSleepingEnabled(false);
    if (world.getBody(other)->isSleeping()) return fail(145);
    world.step(dt);
    return world.lastStepStats().sleepingBodyCount == 0 && world.lastStepStats().solvedContactCount == 3;
}

static bool near(float a, float b, float tol = 1e-5f) { return std::fabs(a - b) <= tol; }

// Bodies built as values (RigidBody::createBox), added with addBody, solved by
// the static SequentialImpulseSolver::solve on a hand-made manifold: a unit
// downward velocity meeting a contact one metre off the centre turns into
// -0.6 m/s down and 0.6 rad/s about z (the known answer of the reference's
// off-centre solver case).
static bool valueBodiesAndStandaloneSolve() {
    RigidBody ground, block;
    std::string error;
    if (!RigidBody::createBox(2.0f, 2.0f, 2.0f, {}, 1.0f, true, 0.0f, 0.0f, ground, error) ||
        !RigidBody::createBox(2.0f, 2.0f, 2.0f, {}, 1.0f, false, 0.0f, 0.0f, block, error))
        return fail(162);
    block.setLinearVelocity({0.0f, -1.0f, 0.0f});
    PhysicsWorld world;
    const RigidBodyHandle a = world.addBody(ground), b = world.addBody(block);
    ContactManifold m{};
    m.bodyA = a;
    m.bodyB = b;
    m.normal = {0.0f, 1.0f, 0.0f};
    m.pointCount = 1;
    m.points[0].localAnchorA = {1.0f, 0.0f, 0.0f};
    m.points[0].localAnchorB = {1.0f, 0.0f, 0.0f};
    std::vector<ContactManifold> contacts{m};
    SequentialImpulseSolver::solve(contacts, world, 1.0f / 60.0f);
    const RigidBody *solved = world.getBody(b);
    const bool ok = solved && near(solved->getLinearVelocity().y, -0.6f) && near(solved->getAngularVelocity().z, 0.6f) &&
                    contacts[0].points[0].normalImpulse > 0.0f && world.lastStepStats().solvedContactCount == 1;
    if (!ok) std::fprintf(stderr, "standalone solve: v.y=%f w.z=%f\n", solved ? solved->getLinearVelocity().y : 0.0f,
                          solved ? solved->getAngularVelocity().z : 0.0f);
    return ok;
}

// Colliders edited through the getCollider pointer and added as values.
static bool colliderEditsAndValueColliders() {
    PhysicsWorld world;
    world.gravity = {};
    RigidBodyHandle left, right;
    ColliderHandle cl, cr;
    std::string error;
    if (!world.createSphere(0.5f, {0, 0, 0}, 1.0f, false, 0, 0.5f, left, cl, error) ||
        !world.createSphere(0.5f, {1.5f, 0, 0}, 1.0f, false, 0, 0.5f, right, cr, error))
        return fail(192);
    world.step(1.0f / 60.0f);
    if (!world.contacts().empty()) return fail(194);
    Collider *c = world.getCollider(cl);
    if (!c || !(c->body == left) || std::get<Sphere>(c->shape).radius != 0.5f) return fail(196);
    c->shape = Sphere{1.2f};  // now reaches the right sphere
    world.step(1.0f / 60.0f);
    if (world.contacts().size() != 1 || std::get<Sphere>(world.getCollider(cl)->shape).radius != 1.2f) return fail(199);
    // a second, offset box collider on the right body
    Collider box;
    box.body = right;
    box.localTransform = Transform({0.0f, 3.0f, 0.0f}, Quaternion::identity());
    box.shape = Box{{0.5f, 0.5f, 0.5f}};
    const ColliderHandle cb = world.addCollider(box);
    const Collider *back = world.getCollider(cb);
    if (!back || !(back->body == right) || std::get<Box>(back->shape).halfExtents.y != 0.5f ||
        back->localTransform.position.y != 3.0f)
        return fail(209);
    box.body = RigidBodyHandle{99, 0};  // stale body: empty handle
    const ColliderHandle none = world.addCollider(box);
    return none.index == 0 && none.generation == 0 && !world.getCollider(ColliderHandle{cb.index, cb.generation + 1});
}

// The stateless statics: broadphase pairs (touching boxes count, lexicographic
// order) and generateContact with the colliders' bodies in the manifold.
static bool statelessStatics() {
    std::vector<Aabb> boxes = {{{0, 0, 0}, {1, 1, 1}}, {{1, 0, 0}, {2, 1, 1}}, {{5, 5, 5}, {6, 6, 6}},
                               {{0.5f, 0.5f, 0.5f}, {0.6f, 0.6f, 0.6f}}};
    BroadPhaseStats st;
    for (BroadPhaseAlgorithm algo : {BroadPhaseAlgorithm::SweepAndPrune, BroadPhaseAlgorithm::UniformGrid}) {
        const std::vector<BroadPhasePair> pairs = BroadPhase::findCandidatePairs(boxes, &st, algo);
        // 0-1 touch at x = 1, 3 lies inside 0; 2 is alone
        if (pairs.size() != 2 || pairs[0].first != 0 || pairs[0].second != 1 || pairs[1].first != 0 ||
            pairs[1].second != 3 || st.aabbPairs != 2)
            return fail(226);
    }
    try {
        BroadPhase::findCandidatePairs(boxes, nullptr, BroadPhaseAlgorithm::DynamicTree);
        return fail(230);
    } catch (const std::invalid_argument &) {
    }
    Collider a, b;
    a.body = {3, 1};
    b.body = {4, 2};
    a.shape = Sphere{0.5f};
    b.shape = Sphere{0.5f};
    ContactManifold m;
    if (!NarrowPhase::generateContact(a, Transform({0, 0, 0}, Quaternion::identity()), b,
                                      Transform({0.8f, 0, 0}, Quaternion::identity()), m))
        return fail(241);
    return m.bodyA == a.body && m.bodyB == b.body && m.pointCount == 1 && near(m.normal.x, 1.0f) &&
           near(m.points[0].penetration, 0.2f);
}

// A pointer taken before steps shows the state after them.
static bool pointerSeesLaterSteps() {
    PhysicsWorld world;
    RigidBodyHandle h;
    ColliderHandle c;
    std::string error;
    if (!world.createSphere(0.5f, {0, 10, 0}, 1.0f, false, 0, 0.5f, h, c, error)) return fail(252);
    const RigidBody *body = world.getBody(h);
    const float y0 = body->getPosition().y;
    for (int i = 0; i < 10; ++i) world.step(1.0f / 60.0f);
    return body->getPosition().y < y0 && body->getLinearVelocity().y < 0.0f;
}

int main() {
    bool ok = boxLandsOnStaticFloor() && tiltedBoxSettlesFlat(1.0f / 60.0f, 0.6f, {0.0f, 0.0f, 1.0f}) &&
              tiltedBoxSettlesFlat(1.0f / 120.0f, 0.9f, {0.6f, 0.0f, 0.8f}) && invalidInputs() &&
              settledStackSleepsAndWakes() && valueBodiesAndStandaloneSolve() && colliderEditsAndValueColliders() &&
              statelessStatics() && pointerSeesLaterSteps();
    std::printf("%s\n", ok ? "facade scenarios ok" : "facade scenarios FAILED");
    return ok ? 0 : 1;
}
