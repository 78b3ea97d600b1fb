/*
 * CPU oracle for the per-step collision-and-contact path of bkuangs/phys-engine's
 * PhysicsWorld::step(dt).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests, the
 * smoke check and the CPU-baseline leg of the benchmark call it to compute the
 * expected answer on the host.  Nothing in the shipped GPU path links, loads or
 * calls it, and it must never be used as a fallback for the GPU path.
 *
 * It is a plain C++ restatement of the reference algorithm, templated on the
 * scalar type (float for bit-exact parity, double for finite differences), with
 * three additions the reference lacks and the GPU path needs:
 *   - a solver iteration count parameter (the reference hard-codes 8,
 *     src/solver/sequential_impulse_solver.cpp:235),
 *   - a solve order given by a manifold permutation (the graph-colour order the
 *     GPU solver uses; the reference solves in manifold order),
 *   - contact feature IDs (the reference has none).
 * Each function in pe_oracle.cpp cites the reference file:line it follows.
 *
 * Parity pin: at 8 iterations and natural order the float instance is checked
 * bit-for-bit against the reference compiled from its own sources (see
 * oracle/Makefile, target `ref`), and against golden fixtures generated from it
 * (tests/golden/).
 */
#ifndef PE_ORACLE_H
#define PE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ow_world ow_world;

/* Manifold record exchanged with the tests (one per contact manifold). */
typedef struct ow_manifold {
    uint32_t body_a_index, body_a_generation;
    uint32_t body_b_index, body_b_generation;
    float normal[3];
    uint32_t point_count;
    float friction;
    float restitution;
    float anchor_a[4][3];
    float anchor_b[4][3];
    float penetration[4];
    float normal_impulse[4];
    float tangent_impulse1[4];
    float tangent_impulse2[4];
    uint32_t feature[4];
} ow_manifold;

typedef struct ow_step_stats {
    uint64_t possible_pairs;
    uint64_t candidate_pairs;
    uint64_t contact_count;
    uint64_t solved_contact_count;
    uint64_t awake_body_count;
    uint64_t sleeping_body_count;
    /* broadphase details */
    uint64_t x_window_comparisons;
    uint64_t aabb_pairs;
    uint64_t grid_comparisons;
    uint64_t grid_entries;
    uint64_t grid_overflow_aabbs;
    double grid_cell_size;
    /* narrowphase details: sphere-sphere, sphere-box, box-box, hull-any */
    uint64_t np_candidates[4];
    uint64_t np_contacts[4];
    /* solver details */
    uint64_t prepared_points;
    uint64_t warm_start_comparisons;
    uint64_t warm_start_matches;
    uint64_t velocity_point_visits;
    uint64_t color_count;
} ow_step_stats;

/* ---- world ---------------------------------------------------------------- */
ow_world *ow_create(int fp64);
ow_world *ow_clone(const ow_world *world);
void ow_destroy(ow_world *world);
void ow_set_gravity(ow_world *world, double gx, double gy, double gz);
/* algo: 0 sweep-and-prune, 1 uniform grid, 2 dynamic tree (the same sorted
   pairs as sweep-and-prune; no sweep counters).  cell_size <= 0 selects the
   reference's median cell size; > 0 fixes the grid cell. */
void ow_set_broadphase(ow_world *world, int algo, double cell_size);
/* order_mode: 0 manifold order (the reference), 1 graph-colour order. */
void ow_set_solver(ow_world *world, int iterations, int order_mode);
void ow_set_threads(ow_world *world, int threads);

/* shape: 0 sphere (dims[0] = radius), 1 box (dims = full width, height, depth).
   Returns 0 on success, nonzero with a message in err otherwise (the reference's
   createSphere/createBox validation).  handles = {body idx, body gen, collider idx,
   collider gen}. */
int ow_create_body(ow_world *world, int shape, const float *dims, const float *pos,
                   float density, int is_static, float restitution, float friction,
                   uint32_t *handles, char *err, int err_len);
/* Convex hull body (project-defined shape): vertices in body space, mass and
   diagonal inverse inertia given by the caller. */
int ow_add_hull_shape(ow_world *world, uint32_t vertex_count, const float *vertices);
int ow_create_hull_body(ow_world *world, int hull_id, const float *pos, float mass,
                        const float *inv_inertia_diag, int is_static, float restitution,
                        float friction, uint32_t *handles);
void ow_remove_body(ow_world *world, uint32_t index, uint32_t generation);
void ow_remove_collider(ow_world *world, uint32_t index, uint32_t generation);
/* addCollider on an existing body: shape 0 sphere (dims[0] radius) or 1 box
   (dims = half extents), local position xyz and rotation xyzw.  Returns 1 for a
   stale body (handle {0, 0}), else 0 with handle = {collider idx, gen}. */
int ow_add_collider(ow_world *world, uint32_t body_index, uint32_t body_generation, int shape, const float *dims,
                    const float *local_pos, const float *local_rot, uint32_t *handle);
/* setSleepingEnabled (physics_world.hpp:63); per-slot isSleeping(); wakeUp();
   applyForce (rigid_body.hpp:53-85).  set_velocity and apply_spin wake the body
   like the reference's velocity setters. */
void ow_set_sleeping_enabled(ow_world *world, int enabled);
void ow_get_sleeping(const ow_world *world, uint8_t *sleeping);
void ow_wake_body(ow_world *world, uint32_t index);
void ow_apply_force(ow_world *world, uint32_t index, const float *force);
uint32_t ow_body_slot_count(const ow_world *world);

/* Per-body state by slot (positions, quaternions xyzw, linear/angular velocity). */
void ow_get_bodies(const ow_world *world, float *pos, float *quat, float *lin, float *ang);
void ow_get_bodies_f64(const ow_world *world, double *pos, double *quat, double *lin, double *ang);
void ow_set_velocity(ow_world *world, uint32_t index, const float *lin, const float *ang);
void ow_set_velocity_f64(ow_world *world, uint32_t index, const double *lin, const double *ang);
/* Body position in the world's precision (finite differences). */
void ow_set_position_f64(ow_world *world, uint32_t index, const double *pos);
/* The reference's orientation idiom: setAngularVelocity(spin); integrateRotation(1);
   setAngularVelocity(0) (tests/solver/sequential_impulse_solver_tests.cpp:349-351). */
void ow_apply_spin(ow_world *world, uint32_t index, const float *spin);
void ow_set_material(ow_world *world, uint32_t index, double mass, double friction,
                     double restitution);
void ow_get_material(const ow_world *world, uint32_t index, double *mass,
                     double *friction, double *restitution);

int ow_step(ow_world *world, float dt);
void ow_get_stats(const ow_world *world, ow_step_stats *stats);
/* Wall time of the last step's stages (ms, 11 values): integrate + bounds,
   broadphase, narrowphase, colouring / order, solve, pose, total; then the
   solve's prepare, warm start, velocity iterations and cache update. */
void ow_get_stage_ms(const ow_world *world, double *ms);
uint32_t ow_pair_count(const ow_world *world);
void ow_get_pairs(const ow_world *world, uint32_t *pairs);
uint32_t ow_contact_count(const ow_world *world);
void ow_get_contacts(const ow_world *world, ow_manifold *out);
/* Solve order and colour per manifold of the last step. */
void ow_get_solve_order(const ow_world *world, uint32_t *order, uint32_t *colors);

/* ---- stateless stages ------------------------------------------------------ */
/* Broadphase over explicit AABBs (float min/max, 3 per box).  Returns the pair
   count; pairs written only if capacity suffices. */
uint64_t ow_broadphase(const float *mins, const float *maxs, uint32_t n, int algo,
                       double cell_size, uint32_t *pairs, uint64_t capacity,
                       ow_step_stats *stats);
/* One narrowphase call (NarrowPhase::generateContact) between two colliders
   given world transforms (pos xyz, quat xyzw).  Returns 1 on contact. */
int ow_generate_contact(int shape_a, const float *dims_a, const float *pos_a,
                        const float *quat_a, int shape_b, const float *dims_b,
                        const float *pos_b, const float *quat_b, ow_manifold *out);
/* SequentialImpulseSolver::solve on the world's bodies with explicit manifolds.
   order == NULL solves in array order. */
void ow_solve(ow_world *world, ow_manifold *contacts, uint32_t count, float dt,
              int iterations, const uint32_t *order, ow_step_stats *stats);
/* Greedy colouring by priority (the GPU's definition) of a manifold list. */
uint32_t ow_color_manifolds(const ow_world *world, const ow_manifold *contacts,
                            uint32_t count, uint32_t *order, uint32_t *colors);

/* GJK/EPA between two support sets given as point clouds in world space
   (intersectGjk / computeEpa).  Returns -1 no intersection, 0 intersecting
   but EPA failed, 1 EPA success (normal, depth). */
int ow_gjk_epa(const float *points_a, uint32_t count_a, const float *points_b,
               uint32_t count_b, float *normal, float *depth, uint32_t *simplex_size);

#ifdef __cplusplus
}
#endif

#endif
