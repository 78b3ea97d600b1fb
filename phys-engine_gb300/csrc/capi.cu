// C ABI (include/phys_gb300.h) over the GPU world.
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>

#include "phys_gb300.h"
#include "batch.h"
#include "rollout.h"
#include "world.h"

struct pe_world {
    std::unique_ptr<pe::World> w;
    uint64_t npWorkers = 1, solverWorkers = 1, bpWorkers = 1;
};

struct pe_batch {
    std::unique_ptr<pe::Batch> b;
};

struct pe_rollout {
    std::unique_ptr<pe::Rollout> r;
};

namespace {

thread_local std::string g_lastError;

pe_status fail(pe_status s, const std::string &msg) {
    g_lastError = msg;
    return s;
}

template <class F> pe_status guarded(F &&f) {
    try {
        return f();
    } catch (const std::invalid_argument &e) {
        return fail(PE_ERR_INVALID_ARGUMENT, e.what());
    } catch (const pe::CudaError &e) {
        return fail(PE_ERR_CUDA, e.what());
    } catch (const std::bad_alloc &e) {
        return fail(PE_ERR_CUDA, e.what());
    } catch (const std::exception &e) {
        return fail(PE_ERR_DEVICE, e.what());
    }
}

// Per-device world for the stateless stage entry points.
std::mutex g_utilMutex;
std::map<int, std::unique_ptr<pe::World>> g_util;
pe::World &utilWorld(int device) {
    auto &slot = g_util[device];
    if (!slot) slot.reset(new pe::World(device));
    return *slot;
}

void fillStats(const pe::StepCounters &c, pe_step_stats *o) {
    std::memset(o, 0, sizeof(*o));
    o->possible_pairs = c.possiblePairs;
    o->candidate_pairs = c.candidatePairs;
    o->contact_count = c.contactCount;
    o->solved_contact_count = c.solvedContactCount;
    o->awake_body_count = c.awakeBodyCount;
    o->sleeping_body_count = c.sleepingBodyCount;
    o->x_window_comparisons = c.xWindow;
    o->aabb_pairs = c.aabbPairs;
    o->grid_comparisons = c.gridComparisons;
    o->grid_entries = c.gridEntries;
    o->grid_overflow_aabbs = c.gridOverflow;
    o->grid_cell_size = c.cellSize;
    for (int k = 0; k < 4; ++k) {
        o->np_candidates[k] = c.npCandidates[k];
        o->np_contacts[k] = c.npContacts[k];
    }
    o->prepared_points = c.preparedPoints;
    o->warm_start_comparisons = c.warmComparisons;
    o->warm_start_matches = c.warmMatches;
    o->velocity_point_visits = c.velocityPointVisits;
    o->color_count = c.colors;
    o->color_rounds = c.colorRounds;
    o->epa_failures = c.epaFailures;
    o->contact_points = c.points;
    o->total_ms = c.gpuMs;
    o->integrate_ms = c.integrateMs;
    o->broadphase_ms = c.broadphaseMs;
    o->narrowphase_ms = c.narrowphaseMs;
    o->solver_ms = c.solverMs;
    o->pose_ms = c.poseMs;
    o->kernel_launches = c.kernelLaunches;
    o->graph_replayed = c.graphed ? 1u : 0u;
}

// RigidBody::createSphere / createBox validation and mass properties
// (src/dynamics/rigid_body.cpp:25-91, src/dynamics/mass_properties.cpp:5-32,
// include/phys/core/constants.hpp:5-16).  Returns an error message or nullptr.
const char *makeBody(int shape, const float *dims, const float *pos, float density, int isStatic, float restitution,
                     float friction, pe::HostBody &b) {
    const float pi = 3.14159265358979323846f;
    const float minSize = 0.01f * 0.01f, maxSize = 64.0f * 64.0f;
    float volume;
    if (shape == PE_SHAPE_SPHERE) {
        float r = dims[0];
        volume = (4.0f / 3.0f) * pi * r * r * r;
        if (volume < minSize) return "Sphere is too small";
        if (volume > maxSize) return "Sphere is too large";
    } else {
        if (dims[0] <= 0.0f || dims[1] <= 0.0f || dims[2] <= 0.0f) return "Box dimensions must be positive";
        volume = dims[0] * dims[1] * dims[2];
        if (volume < minSize) return "Box is too small";
        if (volume > maxSize) return "Box is too large";
    }
    if (!(density >= 0.2f && density <= 21.4f)) return "Density is out of range";
    float rest = restitution;
    if (rest < 0.0f) rest = 0.0f;
    if (rest > 1.0f) rest = 1.0f;
    const float mass = volume * density;
    b = pe::HostBody{};
    b.mass = mass;
    b.restitution = rest;
    b.friction = friction < 0.0f ? 0.0f : friction;
    b.isStatic = isStatic != 0;
    b.pos[0] = pos[0];
    b.pos[1] = pos[1];
    b.pos[2] = pos[2];
    if (!isStatic) {
        if (shape == PE_SHAPE_SPHERE) {
            float r = dims[0];
            if (mass > 0.0f && r > 0.0f) {
                float ii = 1.0f / (0.4f * mass * r * r);
                b.iinv[0] = b.iinv[1] = b.iinv[2] = ii;
            }
        } else if (mass > 0.0f) {
            float w = dims[0], h = dims[1], d = dims[2];
            float factor = 12.0f / mass;
            b.iinv[0] = factor / (h * h + d * d);
            b.iinv[1] = factor / (w * w + d * d);
            b.iinv[2] = factor / (w * w + h * h);
        }
    }
    return nullptr;
}

pe_status createBody(pe_world *world, int shape, const float *dims, const float *pos, float density, int isStatic,
                     float restitution, float friction, pe_handle *body, pe_handle *collider) {
    if (!world || !dims || !pos) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    pe::HostBody b;
    if (const char *err = makeBody(shape, dims, pos, density, isStatic, restitution, friction, b))
        return fail(PE_ERR_CREATE_FAILED, err);
    uint32_t bg, cg;
    uint32_t bi = world->w->addBody(b, bg);
    pe::HostCollider c;
    c.body = bi;
    c.bodyGeneration = bg;
    c.shape = (uint32_t)shape;
    if (shape == PE_SHAPE_SPHERE) {
        c.dims[0] = dims[0];
    } else {
        // PhysicsWorld::createBox stores half extents (physics_world.cpp:218)
        c.dims[0] = dims[0] * 0.5f;
        c.dims[1] = dims[1] * 0.5f;
        c.dims[2] = dims[2] * 0.5f;
    }
    uint32_t ci = world->w->addCollider(c, cg);
    if (body) *body = pe_handle{bi, bg};
    if (collider) *collider = pe_handle{ci, cg};
    return PE_OK;
}

// RigidBody::integrateRotation (src/dynamics/rigid_body.cpp:110-125).
void integrateRotation(pe::HostBody &b, float dt) {
    if (b.isStatic || b.sleeping) return;
    const float wx = b.ang[0], wy = b.ang[1], wz = b.ang[2];
    const float x = b.rot[0], y = b.rot[1], z = b.rot[2], w = b.rot[3];
    const float sw = 0.0f;
    // spin * rotation (quaternion.hpp:24-31)
    float dx = sw * x + wx * w + wy * z - wz * y;
    float dy = sw * y - wx * z + wy * w + wz * x;
    float dz = sw * z + wx * y - wy * x + wz * w;
    float dw = sw * w - wx * x - wy * y - wz * z;
    const float h2 = 0.5f * dt;
    float q[4] = {x + h2 * dx, y + h2 * dy, z + h2 * dz, w + h2 * dw};
    float len = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    if (len == 0.0f) {
        b.rot[0] = b.rot[1] = b.rot[2] = 0.0f;
        b.rot[3] = 1.0f;
    } else {
        for (int k = 0; k < 4; ++k) b.rot[k] = q[k] / len;
    }
}

} // namespace

extern "C" {

const char *pe_last_error(void) { return g_lastError.c_str(); }

int pe_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

pe_status pe_world_create(int device, pe_world **out) {
    if (!out) return fail(PE_ERR_INVALID_ARGUMENT, "null output");
    return guarded([&] {
        auto *w = new pe_world;
        try {
            w->w.reset(new pe::World(device));
        } catch (...) {
            delete w;
            throw;
        }
        *out = w;
        return PE_OK;
    });
}

void pe_world_destroy(pe_world *world) { delete world; }

pe_status pe_world_clone(pe_world *world, pe_world **out) {
    if (!world || !out) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        auto *c = new pe_world;
        try {
            c->w = world->w->clone();
        } catch (...) {
            delete c;
            throw;
        }
        c->npWorkers = world->npWorkers;
        c->solverWorkers = world->solverWorkers;
        c->bpWorkers = world->bpWorkers;
        *out = c;
        return PE_OK;
    });
}

pe_status pe_world_set_gravity(pe_world *world, float x, float y, float z) {
    if (!world) return fail(PE_ERR_INVALID_ARGUMENT, "null world");
    world->w->gravity[0] = x;
    world->w->gravity[1] = y;
    world->w->gravity[2] = z;
    return PE_OK;
}
pe_status pe_world_get_gravity(const pe_world *world, float *xyz) {
    if (!world || !xyz) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    std::memcpy(xyz, world->w->gravity, 3 * sizeof(float));
    return PE_OK;
}
pe_status pe_world_set_broadphase(pe_world *world, int algorithm) {
    if (!world || algorithm < 0 || algorithm > 2) return fail(PE_ERR_INVALID_ARGUMENT, "unknown broadphase algorithm");
    world->w->algorithm = algorithm;
    return PE_OK;
}
pe_status pe_world_get_broadphase(const pe_world *world, int *algorithm) {
    if (!world || !algorithm) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    *algorithm = world->w->algorithm;
    return PE_OK;
}
pe_status pe_world_set_grid_cell_size(pe_world *world, double cell) {
    if (!world || !std::isfinite(cell)) return fail(PE_ERR_INVALID_ARGUMENT, "cell size must be finite");
    world->w->cellSize = cell;
    return PE_OK;
}
pe_status pe_world_set_solver(pe_world *world, int iterations, int order) {
    if (!world || iterations < 0 || (order != PE_ORDER_MANIFOLD && order != PE_ORDER_COLOR))
        return fail(PE_ERR_INVALID_ARGUMENT, "invalid solver settings");
    world->w->iterations = iterations;
    world->w->orderMode = order;
    return PE_OK;
}
pe_status pe_world_set_worker_counts(pe_world *world, uint64_t np, uint64_t solver, uint64_t bp) {
    if (!world) return fail(PE_ERR_INVALID_ARGUMENT, "null world");
    // physics_world.cpp:132-160
    if (np == 0) return fail(PE_ERR_INVALID_ARGUMENT, "Narrowphase worker count must be positive");
    if (solver == 0) return fail(PE_ERR_INVALID_ARGUMENT, "Solver worker count must be positive");
    if (bp == 0) return fail(PE_ERR_INVALID_ARGUMENT, "Broadphase worker count must be positive");
    world->npWorkers = np;
    world->solverWorkers = solver;
    world->bpWorkers = bp;
    return PE_OK;
}
pe_status pe_world_set_sleeping_enabled(pe_world *world, int enabled) {
    if (!world) return fail(PE_ERR_INVALID_ARGUMENT, "null world");
    return guarded([&] {
        world->w->setSleepingEnabled(enabled != 0);
        return PE_OK;
    });
}
pe_status pe_world_get_sleeping_enabled(const pe_world *world, int *enabled) {
    if (!world || !enabled) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    *enabled = world->w->sleepingEnabled ? 1 : 0;
    return PE_OK;
}

pe_status pe_world_create_sphere(pe_world *world, float radius, const float *position, float density, int is_static,
                                 float restitution, float friction, pe_handle *body, pe_handle *collider) {
    float dims[3] = {radius, 0.0f, 0.0f};
    return guarded(
        [&] { return createBody(world, PE_SHAPE_SPHERE, dims, position, density, is_static, restitution, friction, body, collider); });
}

pe_status pe_world_create_box(pe_world *world, float width, float height, float depth, const float *position,
                              float density, int is_static, float restitution, float friction, pe_handle *body,
                              pe_handle *collider) {
    float dims[3] = {width, height, depth};
    return guarded(
        [&] { return createBody(world, PE_SHAPE_BOX, dims, position, density, is_static, restitution, friction, body, collider); });
}

pe_status pe_world_create_hull(pe_world *world, const float *vertices, uint32_t n, const float *position, float mass,
                               const float *iinv, int is_static, float restitution, float friction, pe_handle *body,
                               pe_handle *collider) {
    if (!world || !vertices || n == 0 || n > 255 || !position || !iinv)
        return fail(PE_ERR_INVALID_ARGUMENT, "hull needs 1..255 vertices, a position and an inverse inertia");
    return guarded([&] {
        pe::HostBody b;
        b.mass = mass;
        b.restitution = restitution;
        b.friction = friction;
        b.isStatic = is_static != 0;
        std::memcpy(b.pos, position, 3 * sizeof(float));
        if (!is_static) std::memcpy(b.iinv, iinv, 3 * sizeof(float));
        uint32_t bg, cg;
        uint32_t bi = world->w->addBody(b, bg);
        pe::HostCollider c;
        c.body = bi;
        c.bodyGeneration = bg;
        c.shape = PE_SHAPE_HULL;
        c.hull = (uint32_t)world->w->addHull(vertices, n);
        uint32_t ci = world->w->addCollider(c, cg);
        if (body) *body = pe_handle{bi, bg};
        if (collider) *collider = pe_handle{ci, cg};
        return PE_OK;
    });
}

pe_status pe_world_add_collider(pe_world *world, pe_handle body, int shape, const float *dims, const float *lpos,
                                const float *lrot, pe_handle *collider) {
    if (!world || !dims || (shape != PE_SHAPE_SPHERE && shape != PE_SHAPE_BOX))
        return fail(PE_ERR_INVALID_ARGUMENT, "sphere or box collider expected");
    return guarded([&] {
        world->w->pull();
        // PhysicsWorld::addCollider returns an empty handle for a stale body
        // (physics_world.cpp:276-281).
        if (!world->w->body(body.index, body.generation)) {
            if (collider) *collider = pe_handle{0, 0};
            return fail(PE_ERR_STALE_HANDLE, "stale body handle");
        }
        pe::HostCollider c;
        c.body = body.index;
        c.bodyGeneration = body.generation;
        c.shape = (uint32_t)shape;
        std::memcpy(c.dims, dims, 3 * sizeof(float));
        if (lpos) std::memcpy(c.lpos, lpos, 3 * sizeof(float));
        if (lrot) std::memcpy(c.lrot, lrot, 4 * sizeof(float));
        uint32_t g;
        uint32_t i = world->w->addCollider(c, g);
        if (collider) *collider = pe_handle{i, g};
        return PE_OK;
    });
}

pe_status pe_world_remove_body(pe_world *world, pe_handle body) {
    if (!world) return fail(PE_ERR_INVALID_ARGUMENT, "null world");
    return guarded([&] {
        world->w->removeBody(body.index, body.generation);
        return PE_OK;
    });
}

pe_status pe_world_remove_collider(pe_world *world, pe_handle collider) {
    if (!world) return fail(PE_ERR_INVALID_ARGUMENT, "null world");
    return guarded([&] {
        world->w->removeCollider(collider.index, collider.generation);
        return PE_OK;
    });
}

pe_status pe_world_get_body(pe_world *world, pe_handle h, pe_body_state *out) {
    if (!world || !out) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        world->w->pull();
        pe::HostBody *b = world->w->body(h.index, h.generation);
        if (!b) return fail(PE_ERR_STALE_HANDLE, "stale body handle");
        std::memcpy(out->position, b->pos, sizeof(out->position));
        std::memcpy(out->rotation, b->rot, sizeof(out->rotation));
        std::memcpy(out->linear_velocity, b->lin, sizeof(out->linear_velocity));
        std::memcpy(out->angular_velocity, b->ang, sizeof(out->angular_velocity));
        std::memcpy(out->force, b->force, sizeof(out->force));
        out->mass = b->mass;
        out->restitution = b->restitution;
        out->friction = b->friction;
        out->is_static = b->isStatic ? 1 : 0;
        return PE_OK;
    });
}

pe_status pe_world_set_body(pe_world *world, pe_handle h, const pe_body_state *in) {
    if (!world || !in) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        world->w->pull();
        pe::HostBody *b = world->w->body(h.index, h.generation);
        if (!b) return fail(PE_ERR_STALE_HANDLE, "stale body handle");
        // A changed velocity or force wakes the body like the reference's
        // setters (setLinearVelocity / setAngularVelocity / applyForce,
        // rigid_body.hpp:54-95); pose, mass, material and static-flag edits
        // wake it at the next step like prepareSleeping's comparison.
        if (std::memcmp(b->lin, in->linear_velocity, sizeof(b->lin)) != 0 ||
            std::memcmp(b->ang, in->angular_velocity, sizeof(b->ang)) != 0 ||
            (!in->is_static && std::memcmp(b->force, in->force, sizeof(b->force)) != 0))
            b->wakeUp();
        std::memcpy(b->pos, in->position, sizeof(b->pos));
        std::memcpy(b->rot, in->rotation, sizeof(b->rot));
        std::memcpy(b->lin, in->linear_velocity, sizeof(b->lin));
        std::memcpy(b->ang, in->angular_velocity, sizeof(b->ang));
        // RigidBody::applyForce ignores static bodies (rigid_body.hpp:77-84)
        if (!in->is_static) std::memcpy(b->force, in->force, sizeof(b->force));
        b->mass = in->mass;
        b->restitution = in->restitution;
        b->friction = in->friction;
        b->isStatic = in->is_static != 0;
        world->w->touch();
        return PE_OK;
    });
}

pe_status pe_world_body_is_sleeping(pe_world *world, pe_handle h, int *sleeping) {
    if (!world || !sleeping) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        world->w->pull();
        pe::HostBody *b = world->w->body(h.index, h.generation);
        if (!b) return fail(PE_ERR_STALE_HANDLE, "stale body handle");
        *sleeping = b->isSleeping() ? 1 : 0;
        return PE_OK;
    });
}

pe_status pe_world_body_wake_up(pe_world *world, pe_handle h) {
    if (!world) return fail(PE_ERR_INVALID_ARGUMENT, "null world");
    return guarded([&] {
        world->w->pull();
        pe::HostBody *b = world->w->body(h.index, h.generation);
        if (!b) return fail(PE_ERR_STALE_HANDLE, "stale body handle");
        b->wakeUp();
        world->w->touch();
        return PE_OK;
    });
}

pe_status pe_world_body_apply_force(pe_world *world, pe_handle h, const float *force) {
    if (!world || !force) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        world->w->pull();
        pe::HostBody *b = world->w->body(h.index, h.generation);
        if (!b) return fail(PE_ERR_STALE_HANDLE, "stale body handle");
        // RigidBody::applyForce (rigid_body.hpp:77-85)
        if (!b->isStatic) {
            if (force[0] != 0.0f || force[1] != 0.0f || force[2] != 0.0f) b->wakeUp();
            for (int k = 0; k < 3; ++k) b->force[k] += force[k];
        }
        world->w->touch();
        return PE_OK;
    });
}

pe_status pe_world_body_set_velocity(pe_world *world, pe_handle h, const float *linear, const float *angular) {
    if (!world) return fail(PE_ERR_INVALID_ARGUMENT, "null world");
    return guarded([&] {
        world->w->pull();
        pe::HostBody *b = world->w->body(h.index, h.generation);
        if (!b) return fail(PE_ERR_STALE_HANDLE, "stale body handle");
        // setLinearVelocity / setAngularVelocity wake the body (rigid_body.hpp:59-63, :91-95)
        if (linear) {
            b->wakeUp();
            std::memcpy(b->lin, linear, sizeof(b->lin));
        }
        if (angular) {
            b->wakeUp();
            std::memcpy(b->ang, angular, sizeof(b->ang));
        }
        world->w->touch();
        return PE_OK;
    });
}

pe_status pe_world_read_sleeping(pe_world *world, uint8_t *sleeping) {
    if (!world || !sleeping) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        world->w->pull();
        const auto &bs = world->w->bodies;
        for (size_t i = 0; i < bs.size(); ++i) sleeping[i] = bs[i].alive && bs[i].isSleeping() ? 1 : 0;
        return PE_OK;
    });
}

pe_status pe_world_body_integrate_rotation(pe_world *world, pe_handle h, float dt) {
    if (!world) return fail(PE_ERR_INVALID_ARGUMENT, "null world");
    return guarded([&] {
        world->w->pull();
        pe::HostBody *b = world->w->body(h.index, h.generation);
        if (!b) return fail(PE_ERR_STALE_HANDLE, "stale body handle");
        integrateRotation(*b, dt);
        world->w->touch();
        return PE_OK;
    });
}

// ------------------------------------------------ RigidBody as a value ---
namespace {
void toRecord(const pe::HostBody &b, pe_body_record *out) {
    std::memcpy(out->state.position, b.pos, sizeof(b.pos));
    std::memcpy(out->state.rotation, b.rot, sizeof(b.rot));
    std::memcpy(out->state.linear_velocity, b.lin, sizeof(b.lin));
    std::memcpy(out->state.angular_velocity, b.ang, sizeof(b.ang));
    std::memcpy(out->state.force, b.force, sizeof(b.force));
    out->state.mass = b.mass;
    out->state.restitution = b.restitution;
    out->state.friction = b.friction;
    out->state.is_static = b.isStatic ? 1 : 0;
    std::memcpy(out->inv_inertia, b.iinv, sizeof(b.iinv));
    out->sleeping = b.sleeping ? 1 : 0;
    out->wake_requested = b.wakeRequested ? 1 : 0;
}
void fromRecord(const pe_body_record &r, pe::HostBody &b) {
    std::memcpy(b.pos, r.state.position, sizeof(b.pos));
    std::memcpy(b.rot, r.state.rotation, sizeof(b.rot));
    std::memcpy(b.lin, r.state.linear_velocity, sizeof(b.lin));
    std::memcpy(b.ang, r.state.angular_velocity, sizeof(b.ang));
    std::memcpy(b.force, r.state.force, sizeof(b.force));
    b.mass = r.state.mass;
    b.restitution = r.state.restitution;
    b.friction = r.state.friction;
    b.isStatic = r.state.is_static != 0;
    std::memcpy(b.iinv, r.inv_inertia, sizeof(b.iinv));
    b.sleeping = r.sleeping != 0;
    b.wakeRequested = r.wake_requested != 0;
}
pe_status makeRecord(int shape, const float *dims, const float *pos, float density, int isStatic, float restitution,
                     float friction, pe_body_record *out) {
    if (!dims || !pos || !out) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    pe::HostBody b;
    if (const char *err = makeBody(shape, dims, pos, density, isStatic, restitution, friction, b))
        return fail(PE_ERR_CREATE_FAILED, err);
    toRecord(b, out);
    return PE_OK;
}
} // namespace

pe_status pe_body_make_sphere(float radius, const float *position, float density, int is_static, float restitution,
                              float friction, pe_body_record *out) {
    const float d[3] = {radius, 0.0f, 0.0f};
    return makeRecord(PE_SHAPE_SPHERE, d, position, density, is_static, restitution, friction, out);
}

pe_status pe_body_make_box(float width, float height, float depth, const float *position, float density,
                           int is_static, float restitution, float friction, pe_body_record *out) {
    const float d[3] = {width, height, depth};
    return makeRecord(PE_SHAPE_BOX, d, position, density, is_static, restitution, friction, out);
}

pe_status pe_body_integrate(pe_body_record *body, int stage, const float *gravity, float dt) {
    if (!body || (stage == PE_INTEGRATE_VELOCITY && !gravity)) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    pe::HostBody b;
    fromRecord(*body, b);
    if (b.isStatic || b.sleeping) return PE_OK;
    if (stage == PE_INTEGRATE_VELOCITY) {
        // RigidBody::integrateVelocity (rigid_body.cpp:94-101)
        const float im = b.mass <= 0.0f ? 0.0f : 1.0f / b.mass;
        for (int k = 0; k < 3; ++k) {
            const float acc = gravity[k] + b.force[k] * im;
            b.lin[k] += acc * dt;
        }
    } else if (stage == PE_INTEGRATE_POSITION) {
        // RigidBody::integratePosition (rigid_body.cpp:103-108)
        for (int k = 0; k < 3; ++k) b.pos[k] += b.lin[k] * dt;
    } else if (stage == PE_INTEGRATE_ROTATION) {
        integrateRotation(b, dt);
    } else {
        return fail(PE_ERR_INVALID_ARGUMENT, "unknown integration stage");
    }
    toRecord(b, body);
    return PE_OK;
}

pe_status pe_world_add_body(pe_world *world, const pe_body_record *body, pe_handle *out) {
    if (!world || !body) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        pe::HostBody b;
        fromRecord(*body, b);
        uint32_t g;
        const uint32_t i = world->w->addBody(b, g);
        if (out) *out = pe_handle{i, g};
        return PE_OK;
    });
}

pe_status pe_world_get_body_record(pe_world *world, pe_handle h, pe_body_record *out) {
    if (!world || !out) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        world->w->pull();
        pe::HostBody *b = world->w->body(h.index, h.generation);
        if (!b) return fail(PE_ERR_STALE_HANDLE, "stale body handle");
        toRecord(*b, out);
        return PE_OK;
    });
}

pe_status pe_world_get_collider(pe_world *world, pe_handle h, pe_handle *body, int *shape, float *dims, float *lpos,
                                float *lrot) {
    if (!world) return fail(PE_ERR_INVALID_ARGUMENT, "null world");
    return guarded([&] {
        pe::HostCollider *c = world->w->collider(h.index, h.generation);
        if (!c) return fail(PE_ERR_STALE_HANDLE, "stale collider handle");
        if (body) *body = pe_handle{c->body, c->bodyGeneration};
        if (shape) *shape = (int)c->shape;
        if (dims) std::memcpy(dims, c->dims, sizeof(c->dims));
        if (lpos) std::memcpy(lpos, c->lpos, sizeof(c->lpos));
        if (lrot) std::memcpy(lrot, c->lrot, sizeof(c->lrot));
        return PE_OK;
    });
}

pe_status pe_world_set_collider(pe_world *world, pe_handle h, pe_handle body, int shape, const float *dims,
                                const float *lpos, const float *lrot) {
    if (!world || !dims || !lpos || !lrot || (shape != PE_SHAPE_SPHERE && shape != PE_SHAPE_BOX))
        return fail(PE_ERR_INVALID_ARGUMENT, "sphere or box collider expected");
    return guarded([&] {
        if (!world->w->setCollider(h.index, h.generation, body.index, body.generation, (uint32_t)shape, dims, lpos,
                                   lrot))
            return fail(PE_ERR_STALE_HANDLE, "stale collider handle");
        return PE_OK;
    });
}

pe_status pe_world_create_bodies(pe_world *world, uint32_t n, const uint8_t *shape, const float *dims,
                                 const float *position, const float *density, const uint8_t *is_static,
                                 const float *restitution, const float *friction, const float *linear_velocity,
                                 const float *spin, pe_handle *bodies, pe_handle *colliders, uint32_t *failed_index) {
    if (!world || (n && (!shape || !dims || !position || !density || !is_static || !restitution || !friction)))
        return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        for (uint32_t i = 0; i < n; ++i) {
            if (shape[i] != PE_SHAPE_SPHERE && shape[i] != PE_SHAPE_BOX)
                return fail(PE_ERR_INVALID_ARGUMENT, "sphere or box shapes expected");
            pe_handle b, c;
            pe_status st = createBody(world, shape[i], dims + 3 * (size_t)i, position + 3 * (size_t)i, density[i],
                                      is_static[i], restitution[i], friction[i], &b, &c);
            if (st != PE_OK) {
                if (failed_index) *failed_index = i;
                return st;
            }
            pe::HostBody *hb = world->w->body(b.index, b.generation);
            if (linear_velocity) {
                // RigidBody::setLinearVelocity (rigid_body.hpp:59-63)
                hb->lin[0] = linear_velocity[3 * (size_t)i];
                hb->lin[1] = linear_velocity[3 * (size_t)i + 1];
                hb->lin[2] = linear_velocity[3 * (size_t)i + 2];
            }
            if (spin && (spin[3 * (size_t)i] != 0.0f || spin[3 * (size_t)i + 1] != 0.0f || spin[3 * (size_t)i + 2] != 0.0f)) {
                hb->ang[0] = spin[3 * (size_t)i];
                hb->ang[1] = spin[3 * (size_t)i + 1];
                hb->ang[2] = spin[3 * (size_t)i + 2];
                integrateRotation(*hb, 1.0f);
                hb->ang[0] = hb->ang[1] = hb->ang[2] = 0.0f;
            }
            if (bodies) bodies[i] = b;
            if (colliders) colliders[i] = c;
        }
        world->w->touch();
        return PE_OK;
    });
}

uint32_t pe_world_body_slot_count(pe_world *world) { return world ? (uint32_t)world->w->bodies.size() : 0u; }

pe_status pe_world_read_bodies(pe_world *world, float *pos, float *rot, float *lin, float *ang) {
    if (!world) return fail(PE_ERR_INVALID_ARGUMENT, "null world");
    return guarded([&] {
        world->w->pull();
        const auto &bs = world->w->bodies;
        for (size_t i = 0; i < bs.size(); ++i) {
            if (pos) std::memcpy(pos + 3 * i, bs[i].pos, 3 * sizeof(float));
            if (rot) std::memcpy(rot + 4 * i, bs[i].rot, 4 * sizeof(float));
            if (lin) std::memcpy(lin + 3 * i, bs[i].lin, 3 * sizeof(float));
            if (ang) std::memcpy(ang + 3 * i, bs[i].ang, 3 * sizeof(float));
        }
        return PE_OK;
    });
}

pe_status pe_world_write_forces(pe_world *world, const float *forces, uint32_t n) {
    if (!world || (n && !forces)) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        world->w->writeForces(forces, n);
        return PE_OK;
    });
}

pe_status pe_world_step_io(pe_world *world, const float *forces, uint32_t n, float dt, float *positions,
                           float *rotations) {
    if (!world || (n && !forces)) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        world->w->stepIO(forces, n, dt, positions, rotations);
        return PE_OK;
    });
}

pe_status pe_world_read_poses(pe_world *world, float *positions, float *rotations) {
    if (!world) return fail(PE_ERR_INVALID_ARGUMENT, "null world");
    return guarded([&] {
        world->w->readPoses(positions, rotations);
        return PE_OK;
    });
}

pe_status pe_world_get_stream(pe_world *world, void **stream) {
    if (!world || !stream) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    *stream = (void *)world->w->stream();
    return PE_OK;
}

pe_status pe_world_set_graphs(pe_world *world, int enabled) {
    if (!world) return fail(PE_ERR_INVALID_ARGUMENT, "null world");
    world->w->setGraphsEnabled(enabled != 0);
    return PE_OK;
}

const char *pe_world_graph_error(pe_world *world) { return world ? world->w->graphError().c_str() : ""; }

pe_status pe_world_step(pe_world *world, float dt) {
    if (!world) return fail(PE_ERR_INVALID_ARGUMENT, "null world");
    return guarded([&] {
        world->w->step(dt);
        return PE_OK;
    });
}

pe_status pe_world_get_step_stats(const pe_world *world, pe_step_stats *out) {
    if (!world || !out) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    fillStats(world->w->counters(), out);
    return PE_OK;
}

pe_status pe_world_get_solver_phases(const pe_world *world, double *ms) {
    if (!world || !ms) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    for (int k = 0; k < 8; ++k) ms[k] = world->w->counters().solverPhaseMs[k];
    return PE_OK;
}

pe_status pe_world_get_contacts(pe_world *world, pe_contact_manifold *out, uint32_t capacity, uint32_t *count) {
    if (!world || !count) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        uint32_t m = world->w->manifoldCount();
        *count = m;
        if (!out || capacity < m) return m == 0 ? PE_OK : fail(PE_ERR_CAPACITY, "contact buffer too small");
        world->w->downloadManifolds(out, m);
        return PE_OK;
    });
}

pe_status pe_world_get_candidate_pairs(pe_world *world, uint32_t *pairs, uint32_t capacity, uint32_t *count) {
    if (!world || !count) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        uint32_t p = world->w->pairCount();
        *count = p;
        if (!pairs || capacity < p) return p == 0 ? PE_OK : fail(PE_ERR_CAPACITY, "pair buffer too small");
        world->w->downloadPairs(pairs);
        return PE_OK;
    });
}

pe_status pe_world_get_solve_order(pe_world *world, uint32_t *order, uint32_t *colors, uint32_t capacity,
                                   uint32_t *count) {
    if (!world || !count) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        uint32_t m = world->w->manifoldCount();
        *count = m;
        if (capacity < m) return m == 0 ? PE_OK : fail(PE_ERR_CAPACITY, "order buffer too small");
        world->w->downloadOrder(order, colors);
        return PE_OK;
    });
}

pe_status pe_world_solve(pe_world *world, pe_contact_manifold *contacts, uint32_t count, float dt) {
    if (!world || (count && !contacts)) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        std::vector<float> recs(count * (sizeof(pe_contact_manifold) / sizeof(float)));
        if (count) std::memcpy(recs.data(), contacts, count * sizeof(pe_contact_manifold));
        world->w->solveOnly(recs, count, dt, world->w->iterations, world->w->orderMode);
        if (count) std::memcpy(contacts, recs.data(), count * sizeof(pe_contact_manifold));
        return PE_OK;
    });
}

pe_status pe_broadphase_find_pairs(int device, const float *mins, const float *maxs, uint32_t n, int algorithm,
                                   double cell, uint32_t *pairs, uint64_t capacity, uint64_t *count,
                                   pe_step_stats *stats) {
    if (!count || (n && (!mins || !maxs))) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    if (algorithm == PE_BROADPHASE_TREE)
        return fail(PE_ERR_INVALID_ARGUMENT, "DynamicTree requires a persistent DynamicAabbTree instance");
    if (algorithm != PE_BROADPHASE_SAP && algorithm != PE_BROADPHASE_GRID)
        return fail(PE_ERR_INVALID_ARGUMENT, "unknown broadphase algorithm");
    return guarded([&] {
        std::lock_guard<std::mutex> lock(g_utilMutex);
        pe::World &w = utilWorld(device);
        std::vector<uint32_t> out;
        pe::StepCounters c;
        w.broadphaseOnly(mins, maxs, n, algorithm, cell, out, c);
        *count = out.size() / 2;
        if (stats) fillStats(c, stats);
        if (!pairs || capacity < *count) return *count == 0 ? PE_OK : fail(PE_ERR_CAPACITY, "pair buffer too small");
        if (!out.empty()) std::memcpy(pairs, out.data(), out.size() * sizeof(uint32_t));
        return PE_OK;
    });
}

pe_status pe_generate_contact(int device, int sa, const float *da, const float *pa, const float *ra, int sb,
                              const float *db, const float *pb, const float *rb, pe_contact_manifold *out, int *hit) {
    if (!da || !pa || !ra || !db || !pb || !rb || !out || !hit) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    if ((sa != PE_SHAPE_SPHERE && sa != PE_SHAPE_BOX) || (sb != PE_SHAPE_SPHERE && sb != PE_SHAPE_BOX))
        return fail(PE_ERR_INVALID_ARGUMENT, "sphere or box shapes expected");
    return guarded([&] {
        std::lock_guard<std::mutex> lock(g_utilMutex);
        pe::World &w = utilWorld(device);
        PE_CHECK(cudaSetDevice(device));
        float4 in[6] = {make_float4(da[0], da[1], da[2], (float)sa), make_float4(pa[0], pa[1], pa[2], 0),
                        make_float4(ra[0], ra[1], ra[2], ra[3]),     make_float4(db[0], db[1], db[2], (float)sb),
                        make_float4(pb[0], pb[1], pb[2], 0),         make_float4(rb[0], rb[1], rb[2], rb[3])};
        float4 *dIn = nullptr, *dOut = nullptr;
        PE_CHECK(cudaMalloc(&dIn, sizeof(in)));
        PE_CHECK(cudaMalloc(&dOut, 11 * sizeof(float4)));
        float4 res[11];
        try {
            PE_CHECK(cudaMemcpyAsync(dIn, in, sizeof(in), cudaMemcpyHostToDevice, w.stream()));
            pe::launchGeneratePairs(dIn, dOut, 1, w.stream());
            PE_CHECK(cudaMemcpyAsync(res, dOut, sizeof(res), cudaMemcpyDeviceToHost, w.stream()));
            PE_CHECK(cudaStreamSynchronize(w.stream()));
        } catch (...) {
            cudaFree(dIn);
            cudaFree(dOut);
            throw;
        }
        cudaFree(dIn);
        cudaFree(dOut);
        std::memset(out, 0, sizeof(*out));
        *hit = res[0].w >= 0.0f ? 1 : 0;
        if (!*hit) return PE_OK;
        out->normal[0] = res[0].x;
        out->normal[1] = res[0].y;
        out->normal[2] = res[0].z;
        out->point_count = (uint32_t)res[0].w;
        for (int k = 0; k < 4; ++k) {
            out->anchor_a[k][0] = res[1 + k].x;
            out->anchor_a[k][1] = res[1 + k].y;
            out->anchor_a[k][2] = res[1 + k].z;
            out->penetration[k] = res[1 + k].w;
            out->anchor_b[k][0] = res[5 + k].x;
            out->anchor_b[k][1] = res[5 + k].y;
            out->anchor_b[k][2] = res[5 + k].z;
        }
        std::memcpy(out->feature, &res[9], 4 * sizeof(uint32_t));
        return PE_OK;
    });
}


// ----------------------------------------------------------------- batch ---
pe_status pe_batch_create(int device, uint32_t worldCount, const uint32_t *worldBodies, const uint8_t *shape,
                          const float *dims, const float *position, const float *density, const uint8_t *isStatic,
                          const float *restitution, const float *friction, const float *linearVelocity,
                          const float *spin, pe_batch **out, uint64_t *failedIndex) {
    if (!out || !worldBodies || !shape || !dims || !position || !density || !isStatic || !restitution || !friction)
        return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    return guarded([&] {
        std::vector<uint32_t> counts(worldBodies, worldBodies + worldCount);
        uint64_t total = 0;
        for (uint32_t n : counts) total += n;
        std::vector<pe::HostBody> bodies(total);
        std::vector<pe::HostCollider> colliders(total);
        uint64_t i = 0;
        for (uint32_t w = 0; w < worldCount; ++w) {
            for (uint32_t k = 0; k < counts[w]; ++k, ++i) {
                if (shape[i] != PE_SHAPE_SPHERE && shape[i] != PE_SHAPE_BOX)
                    return fail(PE_ERR_INVALID_ARGUMENT, "sphere or box shapes expected");
                const float *d = dims + 3 * i;
                if (const char *err = makeBody(shape[i], d, position + 3 * i, density[i], isStatic[i],
                                               restitution[i], friction[i], bodies[i])) {
                    if (failedIndex) *failedIndex = i;
                    return fail(PE_ERR_CREATE_FAILED, err);
                }
                pe::HostBody &hb = bodies[i];
                if (linearVelocity) {
                    hb.lin[0] = linearVelocity[3 * i];
                    hb.lin[1] = linearVelocity[3 * i + 1];
                    hb.lin[2] = linearVelocity[3 * i + 2];
                }
                if (spin && (spin[3 * i] != 0.0f || spin[3 * i + 1] != 0.0f || spin[3 * i + 2] != 0.0f)) {
                    hb.ang[0] = spin[3 * i];
                    hb.ang[1] = spin[3 * i + 1];
                    hb.ang[2] = spin[3 * i + 2];
                    integrateRotation(hb, 1.0f);
                    hb.ang[0] = hb.ang[1] = hb.ang[2] = 0.0f;
                }
                pe::HostCollider &c = colliders[i];
                c.body = k;
                c.shape = shape[i];
                if (shape[i] == PE_SHAPE_SPHERE) {
                    c.dims[0] = d[0];
                } else {
                    c.dims[0] = d[0] * 0.5f;
                    c.dims[1] = d[1] * 0.5f;
                    c.dims[2] = d[2] * 0.5f;
                }
            }
        }
        std::unique_ptr<pe_batch> b(new pe_batch);
        b->b.reset(new pe::Batch(device));
        b->b->create(counts, bodies, colliders);
        *out = b.release();
        return PE_OK;
    });
}

void pe_batch_destroy(pe_batch *batch) { delete batch; }

pe_status pe_batch_set_gravity(pe_batch *batch, float x, float y, float z) {
    if (!batch) return fail(PE_ERR_INVALID_ARGUMENT, "null batch");
    batch->b->gravity[0] = x;
    batch->b->gravity[1] = y;
    batch->b->gravity[2] = z;
    batch->b->invalidateGraphs();
    return PE_OK;
}

pe_status pe_batch_set_iterations(pe_batch *batch, int iterations) {
    if (!batch || iterations < 0 || iterations > 4096) return fail(PE_ERR_INVALID_ARGUMENT, "invalid iteration count");
    batch->b->iterations = iterations;
    batch->b->invalidateGraphs();
    return PE_OK;
}

pe_status pe_batch_step(pe_batch *batch, float dt, uint32_t steps) {
    if (!batch) return fail(PE_ERR_INVALID_ARGUMENT, "null batch");
    return guarded([&] {
        for (uint32_t k = 0; k < steps; ++k) batch->b->step(dt);
        return PE_OK;
    });
}

pe_status pe_batch_autotune(pe_batch *batch, float dt, int repetitions) {
    if (!batch) return fail(PE_ERR_INVALID_ARGUMENT, "null batch");
    return guarded([&] {
        batch->b->autotune(dt, repetitions);
        return PE_OK;
    });
}

pe_status pe_batch_bucket_count(pe_batch *batch, uint32_t *count) {
    if (!batch || !count) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    *count = (uint32_t)batch->b->buckets().size();
    return PE_OK;
}

pe_status pe_batch_get_bucket(pe_batch *batch, uint32_t index, pe_batch_bucket *out) {
    if (!batch || !out) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    const auto &bs = batch->b->buckets();
    if (index >= bs.size()) return fail(PE_ERR_INVALID_ARGUMENT, "bucket index out of range");
    const pe::BatchBucket &b = bs[index];
    std::memset(out, 0, sizeof(*out));
    out->min_bodies = b.lo;
    out->max_bodies = b.hi;
    out->world_count = (uint32_t)b.worlds.size();
    out->threads = (uint32_t)pe::kBatchVariants[b.variant].threads;
    out->min_blocks_per_sm = (uint32_t)pe::kBatchVariants[b.variant].minBlocks;
    out->blocks = b.blocks;
    out->tuned_ms = b.tunedMs;
    for (size_t v = 0; v < b.candidateMs.size() && v < 8; ++v) out->candidate_ms[v] = b.candidateMs[v];
    return PE_OK;
}

pe_status pe_batch_body_count(pe_batch *batch, uint64_t *count) {
    if (!batch || !count) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    *count = batch->b->bodyCount();
    return PE_OK;
}

pe_status pe_batch_read_bodies(pe_batch *batch, float *pos, float *rot, float *lin, float *ang) {
    if (!batch) return fail(PE_ERR_INVALID_ARGUMENT, "null batch");
    return guarded([&] {
        batch->b->readBodies(pos, rot, lin, ang);
        return PE_OK;
    });
}

pe_status pe_batch_write_bodies(pe_batch *batch, const float *pos, const float *rot, const float *lin,
                                const float *ang) {
    if (!batch) return fail(PE_ERR_INVALID_ARGUMENT, "null batch");
    return guarded([&] {
        batch->b->writeBodies(pos, rot, lin, ang);
        return PE_OK;
    });
}

pe_status pe_batch_write_forces(pe_batch *batch, const float *forces) {
    if (!batch || !forces) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        batch->b->writeForces(forces);
        return PE_OK;
    });
}

pe_status pe_batch_read_poses(pe_batch *batch, float *pos, float *rot) {
    if (!batch || !pos || !rot) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        batch->b->readPoses(pos, rot);
        return PE_OK;
    });
}

pe_status pe_batch_get_world_stats(pe_batch *batch, uint32_t world, pe_step_stats *out) {
    if (!batch || !out) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        pe::StepCounters c;
        batch->b->worldCounters(world, c);
        fillStats(c, out);
        return PE_OK;
    });
}

pe_status pe_batch_get_world_pairs(pe_batch *batch, uint32_t world, uint32_t *pairs, uint32_t capacity,
                                   uint32_t *count) {
    if (!batch || !count) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        *count = batch->b->worldPairs(world, pairs, capacity);
        if (*count && (!pairs || capacity < *count)) return fail(PE_ERR_CAPACITY, "pair buffer too small");
        return PE_OK;
    });
}

pe_status pe_batch_get_world_contacts(pe_batch *batch, uint32_t world, pe_contact_manifold *out, uint32_t capacity,
                                      uint32_t *count) {
    if (!batch || !count) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    return guarded([&] {
        *count = batch->b->worldManifolds(world, out, capacity);
        if (*count && (!out || capacity < *count)) return fail(PE_ERR_CAPACITY, "contact buffer too small");
        return PE_OK;
    });
}

pe_status pe_batch_get_stream(pe_batch *batch, void **stream) {
    if (!batch || !stream) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    *stream = (void *)batch->b->stream();
    return PE_OK;
}

pe_status pe_batch_set_graphs(pe_batch *batch, int enabled) {
    if (!batch) return fail(PE_ERR_INVALID_ARGUMENT, "null batch");
    batch->b->setGraphsEnabled(enabled != 0);
    return PE_OK;
}


// --------------------------------------------------------------- rollout ---
pe_status pe_rollout_create(int device, uint32_t worldCount, const uint32_t *worldBodies, const uint8_t *shape,
                            const float *dims, const float *density, const uint8_t *isStatic, uint32_t steps,
                            float dt, int iterations, uint32_t checkpointEvery, pe_rollout **out, float *massOut) {
    if (!out || !worldBodies || !shape || !dims || !density || !isStatic)
        return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    return guarded([&] {
        std::vector<uint32_t> counts(worldBodies, worldBodies + worldCount);
        uint64_t total = 0;
        for (uint32_t n : counts) total += n;
        std::vector<uint8_t> sh(shape, shape + total), st(isStatic, isStatic + total);
        std::vector<float> he(3 * total), ii(3 * total);
        for (uint64_t i = 0; i < total; ++i) {
            if (shape[i] != PE_SHAPE_SPHERE && shape[i] != PE_SHAPE_BOX)
                return fail(PE_ERR_INVALID_ARGUMENT, "sphere or box shapes expected");
            pe::HostBody b;
            if (const char *err = makeBody(shape[i], dims + 3 * i, dims + 3 * i, density[i], isStatic[i], 0.0f, 0.0f, b))
                return fail(PE_ERR_CREATE_FAILED, std::string("body ") + std::to_string(i) + ": " + err);
            for (int j = 0; j < 3; ++j) {
                he[3 * i + j] = shape[i] == PE_SHAPE_SPHERE ? dims[3 * i] : dims[3 * i + j] * 0.5f;
                ii[3 * i + j] = b.iinv[j];
            }
            if (massOut) massOut[i] = b.mass;
        }
        std::unique_ptr<pe_rollout> r(new pe_rollout);
        r->r.reset(new pe::Rollout(device));
        r->r->create(counts, sh, st, he, ii, steps, dt, iterations, checkpointEvery);
        *out = r.release();
        return PE_OK;
    });
}

void pe_rollout_destroy(pe_rollout *rollout) { delete rollout; }

pe_status pe_rollout_set_gravity(pe_rollout *rollout, float x, float y, float z) {
    if (!rollout) return fail(PE_ERR_INVALID_ARGUMENT, "null rollout");
    rollout->r->gravity[0] = x;
    rollout->r->gravity[1] = y;
    rollout->r->gravity[2] = z;
    return PE_OK;
}

pe_status pe_rollout_forward(pe_rollout *rollout, const float *x0, const float *q0, const float *v0, const float *w0,
                             const float *mass, const float *friction, const float *restitution, float *xT,
                             float *qT, float *vT, float *wT, void *stream) {
    if (!rollout) return fail(PE_ERR_INVALID_ARGUMENT, "null rollout");
    return guarded([&] {
        rollout->r->forward(x0, q0, v0, w0, mass, friction, restitution, xT, qT, vT, wT,
                            static_cast<cudaStream_t>(stream));
        return PE_OK;
    });
}

pe_status pe_rollout_backward(pe_rollout *rollout, const float *dx, const float *dq, const float *dv, const float *dw,
                              float *dx0, float *dq0, float *dv0, float *dw0, float *dmass, float *dfriction,
                              float *drest, void *stream) {
    if (!rollout) return fail(PE_ERR_INVALID_ARGUMENT, "null rollout");
    return guarded([&] {
        rollout->r->backward(dx, dq, dv, dw, dx0, dq0, dv0, dw0, dmass, dfriction, drest,
                             static_cast<cudaStream_t>(stream));
        return PE_OK;
    });
}

pe_status pe_rollout_timings(pe_rollout *rollout, double *fwd, double *bwd) {
    if (!rollout) return fail(PE_ERR_INVALID_ARGUMENT, "null rollout");
    if (fwd) *fwd = rollout->r->lastForwardMs();
    if (bwd) *bwd = rollout->r->lastBackwardMs();
    return PE_OK;
}

pe_status pe_rollout_set_manifold_capacity(pe_rollout *rollout, float per_body) {
    if (!rollout) return fail(PE_ERR_INVALID_ARGUMENT, "null rollout");
    return guarded([&] {
        rollout->r->setManifoldCapacity(per_body);
        return PE_OK;
    });
}

pe_status pe_rollout_device_bytes(pe_rollout *rollout, uint64_t *bytes) {
    if (!rollout || !bytes) return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    *bytes = rollout->r->deviceBytes();
    return PE_OK;
}

} // extern "C"

namespace pe {
void findPairsNoAlloc(int device, const float *mins, const float *maxs, uint32_t n, uint32_t *pairs,
                      uint32_t capacity, uint32_t *result, cudaStream_t s);
}

pe_status pe_debug_set_spin_limit(int device, uint32_t limit) {
    return guarded([&] {
        int previous = 0;
        PE_CHECK(cudaGetDevice(&previous));
        PE_CHECK(cudaSetDevice(device));
        pe::setSpinLimit(limit);
        PE_CHECK(cudaSetDevice(previous));
        return PE_OK;
    });
}

// Allocation-free SAP query for callers that may not allocate device memory;
// the kernel, its fixed scratch array and the per-device set-up are in noalloc.cu.
extern "C" pe_status pe_broadphase_find_pairs_noalloc(int device, const float *d_mins, const float *d_maxs,
                                                      uint32_t n, uint32_t *d_pairs, uint32_t capacity,
                                                      uint32_t *d_result, void *stream) {
    if (!d_result || (n && (!d_mins || !d_maxs)) || (capacity && !d_pairs))
        return fail(PE_ERR_INVALID_ARGUMENT, "null argument");
    if (n > PE_NOALLOC_MAX_BOXES)
        return fail(PE_ERR_INVALID_ARGUMENT, "pe_broadphase_find_pairs_noalloc: " + std::to_string(n) +
                                                 " boxes exceed its limit of " +
                                                 std::to_string(PE_NOALLOC_MAX_BOXES) +
                                                 " (PE_NOALLOC_MAX_BOXES); use pe_broadphase_find_pairs");
    return guarded([&] {
        pe::findPairsNoAlloc(device, d_mins, d_maxs, n, d_pairs, capacity, d_result,
                             static_cast<cudaStream_t>(stream));
        return PE_OK;
    });
}
