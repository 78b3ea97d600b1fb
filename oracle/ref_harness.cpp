// Reference harness (test infrastructure only): a C API over the UNMODIFIED
// bkuangs/phys-engine library, compiled from its own sources by
// oracle/Makefile (target `ref`) into oracle/_ref/.  It exists only where the
// reference sources are present; it pins the oracle restatement and generates
// the golden fixtures under tests/golden/.  Record layouts are shared with the
// oracle (pe_oracle.h).
#include "pe_oracle.h"

#include <phys/collision/broadphase.hpp>
#include <phys/collision/epa.hpp>
#include <phys/collision/gjk.hpp>
#include <phys/collision/narrowphase.hpp>
#include <phys/solver/sequential_impulse_solver.hpp>
#include <phys/world/physics_world.hpp>

#include <cstring>
#include <string>
#include <vector>

using namespace phys;

struct rw_world {
    PhysicsWorld world;
    std::vector<RigidBodyHandle> bodies;   // by body slot index
    std::vector<ColliderHandle> colliders; // by body slot index (one collider per body)
};

static void toRecord(const ContactManifold &m, ow_manifold &r) {
    std::memset(&r, 0, sizeof(r));
    r.body_a_index = m.bodyA.index;
    r.body_a_generation = m.bodyA.generation;
    r.body_b_index = m.bodyB.index;
    r.body_b_generation = m.bodyB.generation;
    r.normal[0] = m.normal.x;
    r.normal[1] = m.normal.y;
    r.normal[2] = m.normal.z;
    r.point_count = m.pointCount;
    r.friction = m.friction;
    r.restitution = m.restitution;
    for (int i = 0; i < 4; ++i) {
        const ContactPoint &p = m.points[i];
        r.anchor_a[i][0] = p.localAnchorA.x;
        r.anchor_a[i][1] = p.localAnchorA.y;
        r.anchor_a[i][2] = p.localAnchorA.z;
        r.anchor_b[i][0] = p.localAnchorB.x;
        r.anchor_b[i][1] = p.localAnchorB.y;
        r.anchor_b[i][2] = p.localAnchorB.z;
        r.penetration[i] = p.penetration;
        r.normal_impulse[i] = p.normalImpulse;
        r.tangent_impulse1[i] = p.tangentImpulse1;
        r.tangent_impulse2[i] = p.tangentImpulse2;
    }
}

static ContactManifold fromRecord(const ow_manifold &r) {
    ContactManifold m{};
    m.bodyA = {r.body_a_index, r.body_a_generation};
    m.bodyB = {r.body_b_index, r.body_b_generation};
    m.normal = {r.normal[0], r.normal[1], r.normal[2]};
    m.pointCount = r.point_count;
    m.friction = r.friction;
    m.restitution = r.restitution;
    for (int i = 0; i < 4; ++i) {
        ContactPoint &p = m.points[i];
        p.localAnchorA = {r.anchor_a[i][0], r.anchor_a[i][1], r.anchor_a[i][2]};
        p.localAnchorB = {r.anchor_b[i][0], r.anchor_b[i][1], r.anchor_b[i][2]};
        p.penetration = r.penetration[i];
        p.normalImpulse = r.normal_impulse[i];
        p.tangentImpulse1 = r.tangent_impulse1[i];
        p.tangentImpulse2 = r.tangent_impulse2[i];
    }
    return m;
}

static void fillStats(const StepStats &s, ow_step_stats *o) {
    std::memset(o, 0, sizeof(*o));
    o->possible_pairs = s.possiblePairs;
    o->candidate_pairs = s.candidatePairs;
    o->contact_count = s.contactCount;
    o->solved_contact_count = s.solvedContactCount;
    o->awake_body_count = s.awakeBodyCount;
    o->sleeping_body_count = s.sleepingBodyCount;
    const BroadPhaseStats &b = s.broadPhaseDetails;
    o->x_window_comparisons = b.xWindowComparisons;
    o->aabb_pairs = b.aabbPairs;
    o->grid_comparisons = b.gridComparisons;
    o->grid_entries = b.gridEntries;
    o->grid_overflow_aabbs = b.gridOverflowAabbs;
    o->grid_cell_size = b.gridCellSize;
    const NarrowPhaseStats &n = s.narrowPhaseDetails;
    o->np_candidates[0] = n.sphereSphereCandidates;
    o->np_candidates[1] = n.sphereBoxCandidates;
    o->np_candidates[2] = n.boxBoxCandidates;
    o->np_contacts[0] = n.sphereSphereContacts;
    o->np_contacts[1] = n.sphereBoxContacts;
    o->np_contacts[2] = n.boxBoxContacts;
    const SolverStats &v = s.solverDetails;
    o->prepared_points = v.preparedPoints;
    o->warm_start_comparisons = v.warmStartComparisons;
    o->warm_start_matches = v.warmStartMatches;
    o->velocity_point_visits = v.velocityPointVisits;
}

extern "C" {

rw_world *rw_create() { return new rw_world; }
rw_world *rw_clone(const rw_world *w) { return new rw_world(*w); }
void rw_destroy(rw_world *w) { delete w; }
void rw_set_gravity(rw_world *w, float x, float y, float z) { w->world.gravity = {x, y, z}; }
void rw_set_broadphase(rw_world *w, int algo) {
    w->world.broadPhaseAlgorithm = algo == 1   ? BroadPhaseAlgorithm::UniformGrid
                                   : algo == 2 ? BroadPhaseAlgorithm::DynamicTree
                                               : BroadPhaseAlgorithm::SweepAndPrune;
}
void rw_set_workers(rw_world *w, int np, int solver, int bp) {
    w->world.setNarrowPhaseWorkerCount((std::size_t)np);
    w->world.setSolverWorkerCount((std::size_t)solver);
    w->world.setBroadPhaseWorkerCount((std::size_t)bp);
}

int rw_create_body(rw_world *w, int shape, const float *dims, const float *pos, float density, int is_static,
                   float restitution, float friction, uint32_t *handles, char *err, int err_len) {
    RigidBodyHandle b;
    ColliderHandle c;
    std::string msg;
    bool ok = shape == 0
                  ? w->world.createSphere(dims[0], {pos[0], pos[1], pos[2]}, density, is_static != 0, restitution,
                                          friction, b, c, msg)
                  : w->world.createBox(dims[0], dims[1], dims[2], {pos[0], pos[1], pos[2]}, density, is_static != 0,
                                       restitution, friction, b, c, msg);
    if (!ok) {
        if (err && err_len > 0) {
            std::strncpy(err, msg.c_str(), (size_t)err_len - 1);
            err[err_len - 1] = 0;
        }
        return 1;
    }
    if (w->bodies.size() <= b.index) {
        w->bodies.resize(b.index + 1);
        w->colliders.resize(b.index + 1);
    }
    w->bodies[b.index] = b;
    w->colliders[b.index] = c;
    handles[0] = b.index;
    handles[1] = b.generation;
    handles[2] = c.index;
    handles[3] = c.generation;
    return 0;
}

void rw_remove_body(rw_world *w, uint32_t index, uint32_t generation) {
    w->world.removeBody({index, generation});
}

int rw_add_collider(rw_world *w, uint32_t body_index, uint32_t body_generation, int shape, const float *dims,
                    const float *local_pos, const float *local_rot, uint32_t *handle) {
    Collider c{};
    c.body = {body_index, body_generation};
    if (shape == 0) c.shape = Sphere{dims[0]};
    else c.shape = Box{{dims[0], dims[1], dims[2]}};
    c.localTransform = Transform{{local_pos[0], local_pos[1], local_pos[2]},
                                 Quaternion{local_rot[0], local_rot[1], local_rot[2], local_rot[3]}};
    ColliderHandle h = w->world.addCollider(c);
    handle[0] = h.index;
    handle[1] = h.generation;
    return w->world.getCollider(h) ? 0 : 1;
}

void rw_remove_collider(rw_world *w, uint32_t index, uint32_t generation) {
    w->world.removeCollider({index, generation});
}

uint32_t rw_body_slot_count(const rw_world *w) { return (uint32_t)w->bodies.size(); }

void rw_set_sleeping_enabled(rw_world *w, int enabled) { w->world.setSleepingEnabled(enabled != 0); }

void rw_get_sleeping(const rw_world *w, uint8_t *sleeping) {
    for (size_t i = 0; i < w->bodies.size(); ++i) {
        const RigidBody *b = w->world.getBody(w->bodies[i]);
        sleeping[i] = b && b->isSleeping() ? 1 : 0;
    }
}

void rw_wake_body(rw_world *w, uint32_t index) {
    if (RigidBody *b = w->world.getBody(w->bodies[index])) b->wakeUp();
}

void rw_apply_force(rw_world *w, uint32_t index, const float *f) {
    if (RigidBody *b = w->world.getBody(w->bodies[index])) b->applyForce({f[0], f[1], f[2]});
}

void rw_set_material(rw_world *w, uint32_t index, float mass, float friction, float restitution) {
    if (RigidBody *b = w->world.getBody(w->bodies[index])) {
        b->mass = mass;
        b->friction = friction;
        b->restitution = restitution;
    }
}

// Orientation idiom of the reference's own tests
// (tests/solver/sequential_impulse_solver_tests.cpp:349-351).
void rw_apply_spin(rw_world *w, uint32_t index, const float *spin) {
    RigidBody *b = w->world.getBody(w->bodies[index]);
    if (!b) return;
    b->setAngularVelocity({spin[0], spin[1], spin[2]});
    b->integrateRotation(1.0f);
    b->setAngularVelocity({});
}

void rw_set_velocity(rw_world *w, uint32_t index, const float *lin, const float *ang) {
    RigidBody *b = w->world.getBody(w->bodies[index]);
    if (!b) return;
    if (lin) b->setLinearVelocity({lin[0], lin[1], lin[2]});
    if (ang) b->setAngularVelocity({ang[0], ang[1], ang[2]});
}

void rw_get_bodies(const rw_world *w, float *pos, float *quat, float *lin, float *ang) {
    for (size_t i = 0; i < w->bodies.size(); ++i) {
        const RigidBody *b = w->world.getBody(w->bodies[i]);
        if (!b) continue;
        Vec3 p = b->getPosition(), v = b->getLinearVelocity(), a = b->getAngularVelocity();
        Quaternion q = b->getRotation();
        if (pos) { pos[3 * i] = p.x; pos[3 * i + 1] = p.y; pos[3 * i + 2] = p.z; }
        if (quat) { quat[4 * i] = q.x; quat[4 * i + 1] = q.y; quat[4 * i + 2] = q.z; quat[4 * i + 3] = q.w; }
        if (lin) { lin[3 * i] = v.x; lin[3 * i + 1] = v.y; lin[3 * i + 2] = v.z; }
        if (ang) { ang[3 * i] = a.x; ang[3 * i + 1] = a.y; ang[3 * i + 2] = a.z; }
    }
}

// Collider bounds as refreshed by the last step (physics_world.cpp:540-551).
void rw_get_bounds(const rw_world *w, float *mins, float *maxs) {
    for (size_t i = 0; i < w->colliders.size(); ++i) {
        const Collider *c = w->world.getCollider(w->colliders[i]);
        if (!c) continue;
        mins[3 * i] = c->bounds.min.x; mins[3 * i + 1] = c->bounds.min.y; mins[3 * i + 2] = c->bounds.min.z;
        maxs[3 * i] = c->bounds.max.x; maxs[3 * i + 1] = c->bounds.max.y; maxs[3 * i + 2] = c->bounds.max.z;
    }
}

void rw_step(rw_world *w, float dt) { w->world.step(dt); }

void rw_get_stats(const rw_world *w, ow_step_stats *s) { fillStats(w->world.lastStepStats(), s); }

// The reference's own stage timings of its last step (ms): integrate velocity,
// broadphase, narrowphase, solver (prepare, warm start, velocity iterations,
// cache update), integrate pose, total.
void rw_get_stage_ms(const rw_world *w, double *ms) {
    const phys::StepStats &s = w->world.lastStepStats();
    const double v[9] = {s.integrateVelocityMs,        s.broadPhaseMs,                s.narrowPhaseMs,
                         s.solverDetails.prepareMs,    s.solverDetails.warmStartMs,   s.solverDetails.velocityIterationsMs,
                         s.solverDetails.cacheUpdateMs, s.integratePoseMs,            s.totalMs};
    for (int i = 0; i < 9; ++i) ms[i] = v[i];
}

uint32_t rw_contact_count(const rw_world *w) { return (uint32_t)w->world.contacts().size(); }
void rw_get_contacts(const rw_world *w, ow_manifold *out) {
    const auto &cs = w->world.contacts();
    for (size_t i = 0; i < cs.size(); ++i) toRecord(cs[i], out[i]);
}

uint64_t rw_broadphase(const float *mins, const float *maxs, uint32_t n, int algo, uint32_t *pairs,
                       uint64_t capacity, ow_step_stats *stats) {
    std::vector<Aabb> bounds(n);
    for (uint32_t i = 0; i < n; ++i) {
        bounds[i].min = {mins[3 * i], mins[3 * i + 1], mins[3 * i + 2]};
        bounds[i].max = {maxs[3 * i], maxs[3 * i + 1], maxs[3 * i + 2]};
    }
    BroadPhaseStats st{};
    auto out = BroadPhase::findCandidatePairs(
        bounds, &st, algo == 1 ? BroadPhaseAlgorithm::UniformGrid : BroadPhaseAlgorithm::SweepAndPrune);
    if (stats) {
        StepStats s{};
        s.broadPhaseDetails = st;
        fillStats(s, stats);
    }
    if (pairs && out.size() <= capacity)
        for (size_t i = 0; i < out.size(); ++i) {
            pairs[2 * i] = (uint32_t)out[i].first;
            pairs[2 * i + 1] = (uint32_t)out[i].second;
        }
    return out.size();
}

int rw_generate_contact(int sa, const float *da, const float *pa, const float *qa, int sb, const float *db,
                        const float *pb, const float *qb, ow_manifold *out) {
    Collider a{}, b{};
    if (sa == 0) a.shape = Sphere{da[0]}; else a.shape = Box{{da[0], da[1], da[2]}};
    if (sb == 0) b.shape = Sphere{db[0]}; else b.shape = Box{{db[0], db[1], db[2]}};
    Transform tA{{pa[0], pa[1], pa[2]}, Quaternion{qa[0], qa[1], qa[2], qa[3]}};
    Transform tB{{pb[0], pb[1], pb[2]}, Quaternion{qb[0], qb[1], qb[2], qb[3]}};
    ContactManifold m{};
    bool hit = NarrowPhase::generateContact(a, tA, b, tB, m);
    toRecord(m, *out);
    return hit ? 1 : 0;
}

// SequentialImpulseSolver::solve fed the manifolds in the given order.
void rw_solve(rw_world *w, ow_manifold *contacts, uint32_t count, float dt, const uint32_t *order,
              ow_step_stats *stats) {
    std::vector<ContactManifold> cs;
    cs.reserve(count);
    for (uint32_t k = 0; k < count; ++k) cs.push_back(fromRecord(contacts[order ? order[k] : k]));
    SequentialImpulseSolver::solve(cs, w->world, dt);
    for (uint32_t k = 0; k < count; ++k) toRecord(cs[k], contacts[order ? order[k] : k]);
    if (stats) fillStats(w->world.lastStepStats(), stats);
}

int rw_gjk_epa(const float *points_a, uint32_t count_a, const float *points_b, uint32_t count_b, float *normal,
               float *depth, uint32_t *simplex_size) {
    std::vector<Vec3> A(count_a), B(count_b);
    for (uint32_t i = 0; i < count_a; ++i) A[i] = {points_a[3 * i], points_a[3 * i + 1], points_a[3 * i + 2]};
    for (uint32_t i = 0; i < count_b; ++i) B[i] = {points_b[3 * i], points_b[3 * i + 1], points_b[3 * i + 2]};
    auto support = [](const std::vector<Vec3> &pts) {
        return [&pts](const Vec3 &d) {
            size_t best = 0;
            float bd = Math3d::dot(pts[0], d);
            for (size_t i = 1; i < pts.size(); ++i) {
                float v = Math3d::dot(pts[i], d);
                if (v > bd) { bd = v; best = i; }
            }
            return pts[best];
        };
    };
    SupportFunction sa = support(A), sb = support(B);
    GjkSimplex s;
    bool hit = intersectGjk(sa, sb, &s);
    if (simplex_size) *simplex_size = s.size;
    if (!hit) return -1;
    EpaResult r;
    bool ok = computeEpa(sa, sb, s, r);
    if (normal) { normal[0] = r.normal.x; normal[1] = r.normal.y; normal[2] = r.normal.z; }
    if (depth) *depth = r.depth;
    return ok ? 1 : 0;
}

} // extern "C"
