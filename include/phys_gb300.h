/*
 * phys-engine-gb300 — C ABI of the GPU collision-and-contact path.
 *
 * Drop-in boundary for bkuangs/phys-engine's PhysicsWorld::step(dt) hot path
 * (src/world/physics_world.cpp:518-782).  The reference exposes C++ classes
 * only; each entry point below names the reference member it replaces.  Plain
 * pointers and sizes only; all device memory is owned by the library.
 *
 * Errors: every function returns a pe_status; pe_last_error() holds the
 * message of the calling thread's last failure.  Reference exceptions map to
 * PE_ERR_INVALID_ARGUMENT, factory `false` returns to PE_ERR_CREATE_FAILED,
 * and `nullptr` from getBody/getCollider to PE_ERR_STALE_HANDLE.
 *
 * Threading: a world is used from one host thread at a time (the reference
 * world is not thread-safe either); each world owns one CUDA stream.
 */
#ifndef PHYS_GB300_H
#define PHYS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum pe_status {
    PE_OK = 0,
    PE_ERR_INVALID_ARGUMENT = 1, /* the reference throws std::invalid_argument */
    PE_ERR_CREATE_FAILED = 2,    /* createSphere/createBox returned false */
    PE_ERR_STALE_HANDLE = 3,     /* getBody/getCollider returned nullptr */
    PE_ERR_CAPACITY = 4,         /* caller buffer too small; *count holds the size needed */
    PE_ERR_UNSUPPORTED = 5,      /* an option outside the GPU path */
    PE_ERR_CUDA = 6,             /* CUDA runtime failure (no device, out of memory, ...) */
    PE_ERR_DEVICE = 7            /* device-side failure: a bounded wait timed out, colour overflow */
} pe_status;

/* BroadPhaseAlgorithm (include/phys/collision/broadphase.hpp:8-13) */
enum { PE_BROADPHASE_SAP = 0, PE_BROADPHASE_GRID = 1, PE_BROADPHASE_TREE = 2 };
/* Collider shapes: Sphere, Box (include/phys/collision/collider.hpp:27) and a
   convex hull (absent from the reference, which only forward-declares one). */
enum { PE_SHAPE_SPHERE = 0, PE_SHAPE_BOX = 1, PE_SHAPE_HULL = 2 };
/* Solver order: the reference's manifold order (one manifold at a time) or the
   GPU's graph-colour order. */
enum { PE_ORDER_MANIFOLD = 0, PE_ORDER_COLOR = 1 };

/* RigidBodyHandle / ColliderHandle (include/phys/world/body_handle.hpp:6-15,
   include/phys/collision/collider.hpp:12-16) */
typedef struct pe_handle {
    uint32_t index;
    uint32_t generation;
} pe_handle;

/* Public RigidBody state (include/phys/dynamics/rigid_body.hpp:14-140). */
typedef struct pe_body_state {
    float position[3];
    float rotation[4]; /* quaternion x, y, z, w */
    float linear_velocity[3];
    float angular_velocity[3];
    float force[3];
    float mass;
    float restitution;
    float friction;
    int32_t is_static;
} pe_body_state;

/* ContactManifold + ContactPoint (include/phys/collision/manifold.hpp:9-34) with
   per-point feature ids added.  216 bytes. */
typedef struct pe_contact_manifold {
    uint32_t body_a_index, body_a_generation;
    uint32_t body_b_index, body_b_generation;
    float normal[3]; /* from body A toward body B */
    uint32_t point_count;
    float friction;
    float restitution;
    float anchor_a[4][3]; /* localAnchorA per point (body A space) */
    float anchor_b[4][3]; /* localAnchorB per point (body B space) */
    float penetration[4];
    float normal_impulse[4];
    float tangent_impulse1[4];
    float tangent_impulse2[4];
    uint32_t feature[4]; /* (kind << 24) | (source << 16) | (face axis << 8) | (face sign << 4) | vertex */
} pe_contact_manifold;

/* StepStats with BroadPhaseStats / NarrowPhaseStats / SolverStats counters
   (include/phys/world/step_stats.hpp:7-54, broadphase.hpp:21-42).  Stage
   timings are replaced by the device time of the whole step. */
typedef struct pe_step_stats {
    uint64_t possible_pairs;
    uint64_t candidate_pairs;
    uint64_t contact_count;
    uint64_t solved_contact_count;
    uint64_t awake_body_count;
    uint64_t sleeping_body_count;
    uint64_t x_window_comparisons;
    uint64_t aabb_pairs;
    uint64_t grid_comparisons;
    uint64_t grid_entries;
    uint64_t grid_overflow_aabbs;
    double grid_cell_size;
    uint64_t np_candidates[4]; /* sphere-sphere, sphere-box, box-box, hull-any */
    uint64_t np_contacts[4];
    uint64_t prepared_points;
    uint64_t warm_start_comparisons;
    uint64_t warm_start_matches;
    uint64_t velocity_point_visits;
    uint64_t color_count;
    uint64_t color_rounds;
    uint64_t epa_failures;
    uint64_t contact_points;
    double total_ms; /* device time of the step: integrate kernel start to pose kernel end */
    /* device time per stage, the GPU counterpart of StepStats::integrateVelocityMs,
       broadPhaseMs, narrowPhaseMs, solverMs, integratePoseMs */
    double integrate_ms;
    double broadphase_ms;
    double narrowphase_ms;
    double solver_ms;
    double pose_ms;
    uint64_t kernel_launches; /* engine kernels launched by the step */
    uint64_t graph_replayed;  /* 1 if the step ran from a captured CUDA graph */
} pe_step_stats;

typedef struct pe_world pe_world;

const char *pe_last_error(void);
/* Library / device check: number of CUDA devices visible. */
int pe_device_count(void);

/* PhysicsWorld::PhysicsWorld() / ~PhysicsWorld() (physics_world.hpp:24-25) */
pe_status pe_world_create(int device, pe_world **out);
void pe_world_destroy(pe_world *world);
/* The PhysicsWorld copy constructor (physics_world.hpp:28, physics_world.cpp:74-93):
   an independent world on the same device with the same bodies, colliders,
   settings, last contacts, candidate pairs, warm-start cache, step counters and
   sleep state; stepping either leaves the other unchanged. */
pe_status pe_world_clone(pe_world *world, pe_world **out);

/* PhysicsWorld::gravity (physics_world.hpp:37) */
pe_status pe_world_set_gravity(pe_world *world, float x, float y, float z);
pe_status pe_world_get_gravity(const pe_world *world, float *xyz);
/* PhysicsWorld::broadPhaseAlgorithm (physics_world.hpp:38).  DynamicTree
   builds a linear BVH over the colliders every step; it reports the pair set
   the reference's incremental tree reports (every tight-AABB overlap, sorted),
   without its tree-maintenance counters. */
pe_status pe_world_set_broadphase(pe_world *world, int algorithm);
pe_status pe_world_get_broadphase(const pe_world *world, int *algorithm);
/* Grid cell size: <= 0 keeps the reference's median policy
   (src/collision/broadphase.cpp:98-110); > 0 fixes it.  No reference counterpart. */
pe_status pe_world_set_grid_cell_size(pe_world *world, double cell_size);
/* Solver iteration count (the reference hard-codes 8,
   src/solver/sequential_impulse_solver.cpp:235) and order (PE_ORDER_*). */
pe_status pe_world_set_solver(pe_world *world, int iterations, int order);
/* setNarrowPhaseWorkerCount / setSolverWorkerCount / setBroadPhaseWorkerCount
   (physics_world.hpp:66-73): validated like the reference (0 is invalid); the
   GPU path has no host worker threads. */
pe_status pe_world_set_worker_counts(pe_world *world, uint64_t narrowphase, uint64_t solver, uint64_t broadphase);
/* setSleepingEnabled / isSleepingEnabled (physics_world.hpp:63-64): islands
   whose bodies stay below 0.05 m/s and 0.05 rad/s for half a second of
   simulated time sleep (no gravity, no solve, fixed pose) until a contact, an
   edit or a wake request wakes them (src/world/physics_world.cpp:341-516). */
pe_status pe_world_set_sleeping_enabled(pe_world *world, int enabled);
pe_status pe_world_get_sleeping_enabled(const pe_world *world, int *enabled);

/* createSphere / createBox (physics_world.hpp:43-50): same validation and mass
   properties as RigidBody::createSphere / createBox (src/dynamics/rigid_body.cpp:25-91). */
pe_status pe_world_create_sphere(pe_world *world, float radius, const float *position, float density,
                                 int is_static, float restitution, float friction, pe_handle *body,
                                 pe_handle *collider);
pe_status pe_world_create_box(pe_world *world, float width, float height, float depth, const float *position,
                              float density, int is_static, float restitution, float friction, pe_handle *body,
                              pe_handle *collider);
/* Bulk creation of n sphere/box bodies, each exactly as createSphere/createBox
   followed by setLinearVelocity(linear_velocity) and the reference's
   orientation idiom setAngularVelocity(spin); integrateRotation(1);
   setAngularVelocity(0) (tests/solver/sequential_impulse_solver_tests.cpp:349-351).
   dims: radius or width/height/depth per body; linear_velocity and spin may be
   NULL.  On a validation failure returns PE_ERR_CREATE_FAILED with the failing
   index in *failed_index; bodies before it stay created.  No reference counterpart. */
pe_status pe_world_create_bodies(pe_world *world, uint32_t n, const uint8_t *shape, const float *dims,
                                 const float *position, const float *density, const uint8_t *is_static,
                                 const float *restitution, const float *friction, const float *linear_velocity,
                                 const float *spin, pe_handle *bodies, pe_handle *colliders, uint32_t *failed_index);
/* Convex hull body (no reference counterpart): vertices in body space, mass and
   diagonal inverse inertia supplied by the caller. */
pe_status pe_world_create_hull(pe_world *world, const float *vertices, uint32_t vertex_count,
                               const float *position, float mass, const float *inverse_inertia, int is_static,
                               float restitution, float friction, pe_handle *body, pe_handle *collider);
/* addCollider (physics_world.hpp:57) for an existing body, with a local
   transform: dims = sphere radius or box half extents; local_position (xyz) and
   local_rotation (xyzw) may be NULL (identity).  A body may hold several
   colliders; pairs of colliders on one body are never candidates. */
pe_status pe_world_add_collider(pe_world *world, pe_handle body, int shape, const float *dims,
                                const float *local_position, const float *local_rotation, pe_handle *collider);
/* removeBody / removeCollider (physics_world.hpp:41, 58) */
pe_status pe_world_remove_body(pe_world *world, pe_handle body);
pe_status pe_world_remove_collider(pe_world *world, pe_handle collider);

/* getBody (physics_world.hpp:54-55) read / write of the public state.  With
   sleeping on, a changed velocity or force wakes the body at once (the
   reference's setters); a changed pose, mass, material or static flag wakes it
   at the next step (prepareSleeping's comparison). */
pe_status pe_world_get_body(pe_world *world, pe_handle body, pe_body_state *out);
pe_status pe_world_set_body(pe_world *world, pe_handle body, const pe_body_state *state);
/* RigidBody::isSleeping / wakeUp / applyForce / setLinearVelocity +
   setAngularVelocity (rigid_body.hpp:53-95); NULL leaves a velocity as it is. */
pe_status pe_world_body_is_sleeping(pe_world *world, pe_handle body, int *sleeping);
pe_status pe_world_body_wake_up(pe_world *world, pe_handle body);
pe_status pe_world_body_apply_force(pe_world *world, pe_handle body, const float *force);
pe_status pe_world_body_set_velocity(pe_world *world, pe_handle body, const float *linear, const float *angular);
/* RigidBody as a value (include/phys/dynamics/rigid_body.hpp:14-140): the public
   state, the diagonal local inverse inertia (inverseInertiaLocal, private in the
   reference and set only by its factories) and the sleep flags (sleeping,
   wakeRequested). */
typedef struct pe_body_record {
    pe_body_state state;
    float inv_inertia[3];
    int32_t sleeping;
    int32_t wake_requested;
} pe_body_record;
/* RigidBody::createSphere / createBox (src/dynamics/rigid_body.cpp:25-92) on the
   host, no world involved: validation (PE_ERR_CREATE_FAILED with the reference's
   message), mass = volume x density, inverse inertia. */
pe_status pe_body_make_sphere(float radius, const float *position, float density, int is_static, float restitution,
                              float friction, pe_body_record *out);
pe_status pe_body_make_box(float width, float height, float depth, const float *position, float density,
                           int is_static, float restitution, float friction, pe_body_record *out);
/* RigidBody::integrateVelocity / integratePosition / integrateRotation
   (rigid_body.cpp:94-125) on a body value; no-ops for static or sleeping bodies. */
enum { PE_INTEGRATE_VELOCITY = 0, PE_INTEGRATE_POSITION = 1, PE_INTEGRATE_ROTATION = 2 };
pe_status pe_body_integrate(pe_body_record *body, int stage, const float *gravity, float dt);
/* PhysicsWorld::addBody (physics_world.cpp:162-179): a body without colliders;
   it enters awake (the reference calls wakeUp). */
pe_status pe_world_add_body(pe_world *world, const pe_body_record *body, pe_handle *out);
/* PhysicsWorld::getBody as a value, sleep flags included. */
pe_status pe_world_get_body_record(pe_world *world, pe_handle body, pe_body_record *out);
/* PhysicsWorld::getCollider (physics_world.cpp:315-339): the collider's body,
   shape, dims (radius / half extents) and local transform; any output may be NULL. */
pe_status pe_world_get_collider(pe_world *world, pe_handle collider, pe_handle *body, int *shape, float *dims,
                                float *lpos, float *lrot);
/* A write through the reference's Collider* (its fields are public): new body,
   shape and local transform of a live collider.  A change of geometry wakes the
   old and the new body, as prepareSleeping's collider comparison does
   (physics_world.cpp:455-465); the device copy is refreshed before the next step. */
pe_status pe_world_set_collider(pe_world *world, pe_handle collider, pe_handle body, int shape, const float *dims,
                                const float *lpos, const float *lrot);
/* isSleeping() of every body slot (0 for empty slots).  No reference counterpart. */
pe_status pe_world_read_sleeping(pe_world *world, uint8_t *sleeping);
/* RigidBody::integrateRotation (rigid_body.cpp:110-125) on one body; with
   dt = 1 and an angular velocity this is the reference's orientation idiom. */
pe_status pe_world_body_integrate_rotation(pe_world *world, pe_handle body, float dt);

/* Bulk state by body slot (positions xyz, quaternions xyzw, linear and angular
   velocity xyz); any pointer may be NULL.  No reference counterpart. */
uint32_t pe_world_body_slot_count(pe_world *world);
pe_status pe_world_read_bodies(pe_world *world, float *positions, float *rotations, float *linear,
                               float *angular);

/* Per-step host I/O without the host mirror (no reference counterpart; the
   reference's equivalents are RigidBody::applyForce and getPosition/getRotation
   per body): set the accumulated force of body slots [0, n) from xyz triples
   (static bodies ignore it, like applyForce, and a nonzero force wakes its
   body), and copy all current positions
   (xyz) / rotations (xyzw) out.  Either output pointer may be NULL. */
pe_status pe_world_write_forces(pe_world *world, const float *forces, uint32_t n);
pe_status pe_world_read_poses(pe_world *world, float *positions, float *rotations);
/* pe_world_write_forces + pe_world_step + pe_world_read_poses in one call with a
   single host-device synchronisation: the forces (n xyz triples, may be 0 / NULL)
   are copied in, the step runs, and the new positions / rotations (either may
   be NULL) are copied out.  Results are those of the three calls. */
pe_status pe_world_step_io(pe_world *world, const float *forces, uint32_t n, float dt, float *positions,
                           float *rotations);
/* The CUDA stream (cudaStream_t) the world's kernels run on, for event timing
   by the caller. */
pe_status pe_world_get_stream(pe_world *world, void **stream);

/* CUDA-graph replay of the step (default on).  Off launches the same kernels
   one by one; results are identical.  No reference counterpart. */
pe_status pe_world_set_graphs(pe_world *world, int enabled);
/* Last graph capture problem of the world (empty when none), for diagnostics. */
const char *pe_world_graph_error(pe_world *world);

/* PhysicsWorld::step (physics_world.hpp:75) */
pe_status pe_world_step(pe_world *world, float dt);
/* lastStepStats (physics_world.hpp:77) */
pe_status pe_world_get_step_stats(const pe_world *world, pe_step_stats *out);
/* Device time (ms) of the phases of the last step's one-cluster contact
   solver, 8 values: the gap from the narrowphase's end to the prepare
   kernel's start, the prepare kernel (prepare, manifold flags, island
   unions), the gap to the cluster kernel's start, island lists, island plan +
   staging (colouring on the colour-phase path), sweeps (island path: with
   each warp's results and cache entries; colour-phase path: with the
   staging), write-back and cache rebuild (colour-phase path only), the gap
   from the solver's end to the pose kernel's start; zeros when the step
   solved on another path.  No reference counterpart (profiling). */
pe_status pe_world_get_solver_phases(const pe_world *world, double *ms);
/* contacts() (physics_world.hpp:61): manifolds of the last step in candidate
   pair order with their solved impulses. */
pe_status pe_world_get_contacts(pe_world *world, pe_contact_manifold *out, uint32_t capacity, uint32_t *count);
/* Candidate collider-slot pairs of the last step (lexicographic), as the
   broadphase + same-body filter produce them (physics_world.cpp:620-633). */
pe_status pe_world_get_candidate_pairs(pe_world *world, uint32_t *pairs, uint32_t capacity, uint32_t *count);
/* Solve order of the last step: order[k] = manifold index solved k-th,
   colors[m] = colour of manifold m. */
pe_status pe_world_get_solve_order(pe_world *world, uint32_t *order, uint32_t *colors, uint32_t capacity,
                                   uint32_t *count);

/* SequentialImpulseSolver::solve(contacts, world, dt)
   (include/phys/solver/sequential_impulse_solver.hpp:17): solves the given
   manifolds against the world's bodies with the world's solver settings,
   writing impulses back into `contacts` and updating the warm-start cache. */
pe_status pe_world_solve(pe_world *world, pe_contact_manifold *contacts, uint32_t count, float dt);

/* BroadPhase::findCandidatePairs (include/phys/collision/broadphase.hpp:52-54):
   mins/maxs are n xyz triples; pairs receives 2*count indices in lexicographic
   order (first < second); stats may be NULL. */
pe_status pe_broadphase_find_pairs(int device, const float *mins, const float *maxs, uint32_t n, int algorithm,
                                   double cell_size, uint32_t *pairs, uint64_t capacity, uint64_t *count,
                                   pe_step_stats *stats);
/* NarrowPhase::generateContact (include/phys/collision/narrowphase.hpp:34-39)
   for sphere/box colliders given world transforms (position xyz, rotation
   xyzw); dims = radius or half extents.  *hit = 1 when a manifold is produced. */
pe_status pe_generate_contact(int device, int shape_a, const float *dims_a, const float *pos_a, const float *rot_a,
                              int shape_b, const float *dims_b, const float *pos_b, const float *rot_b,
                              pe_contact_manifold *out, int *hit);

/* ------------------------------------------------------------------------
   Batched worlds.  The reference steps one PhysicsWorld at a time; a batch
   holds many independent worlds and steps all of them with one persistent
   kernel launch per world-size bucket, captured in one CUDA graph per step.
   Each world behaves as a PhysicsWorld (physics_world.hpp:21-153) of sphere and
   box bodies, one collider each, with the SAP broadphase and the graph-colour
   solve order, and gives the same results as a pe_world holding the same
   bodies.  Limits: <= 8192 bodies and <= 4096 contact manifolds per world.
   ------------------------------------------------------------------------ */
typedef struct pe_batch pe_batch;

typedef struct pe_batch_bucket {
    uint32_t min_bodies, max_bodies; /* world sizes in this bucket */
    uint32_t world_count;
    uint32_t threads;                /* kernel variant: threads per block ... */
    uint32_t min_blocks_per_sm;      /* ... and the residency its registers are sized for */
    uint32_t blocks;                 /* persistent blocks launched */
    double tuned_ms;                 /* autotuner's time per launch; 0 = not tuned */
    double candidate_ms[8];          /* per kernel variant; -1 = does not fit, 0 = not timed */
} pe_batch_bucket;

/* world_body_counts[w] bodies per world; the per-body arrays hold all worlds'
   bodies back to back, with the meaning of pe_world_create_bodies (shapes
   sphere or box; linear_velocity and spin may be NULL).  On a validation
   failure returns PE_ERR_CREATE_FAILED with the failing body in *failed_index. */
pe_status pe_batch_create(int device, uint32_t world_count, const uint32_t *world_body_counts, const uint8_t *shape,
                          const float *dims, const float *position, const float *density, const uint8_t *is_static,
                          const float *restitution, const float *friction, const float *linear_velocity,
                          const float *spin, pe_batch **out, uint64_t *failed_index);
void pe_batch_destroy(pe_batch *batch);
pe_status pe_batch_set_gravity(pe_batch *batch, float x, float y, float z);
/* Solver velocity iterations of every world (the reference's fixed 8 by default). */
pe_status pe_batch_set_iterations(pe_batch *batch, int iterations);
/* `steps` steps of every world (PhysicsWorld::step(dt) per world). */
pe_status pe_batch_step(pe_batch *batch, float dt, uint32_t steps);
/* Times every kernel variant on every bucket (`repetitions` launches each,
   from the current state, which stays unchanged) and keeps the fastest. */
pe_status pe_batch_autotune(pe_batch *batch, float dt, int repetitions);
pe_status pe_batch_bucket_count(pe_batch *batch, uint32_t *count);
pe_status pe_batch_get_bucket(pe_batch *batch, uint32_t index, pe_batch_bucket *out);
pe_status pe_batch_body_count(pe_batch *batch, uint64_t *count);
/* All bodies, world by world (positions/linear/angular xyz, rotations xyzw);
   any pointer may be NULL. */
pe_status pe_batch_read_bodies(pe_batch *batch, float *positions, float *rotations, float *linear, float *angular);
pe_status pe_batch_write_bodies(pe_batch *batch, const float *positions, const float *rotations,
                                const float *linear, const float *angular);
/* Per-body force for the next step, from host memory (RigidBody::applyForce;
   like PhysicsWorld::step, the step clears it afterwards). */
pe_status pe_batch_write_forces(pe_batch *batch, const float *forces);
pe_status pe_batch_read_poses(pe_batch *batch, float *positions, float *rotations);
/* Last step's StepStats, candidate pairs and contacts of one world (body
   indices within the world). */
pe_status pe_batch_get_world_stats(pe_batch *batch, uint32_t world, pe_step_stats *out);
pe_status pe_batch_get_world_pairs(pe_batch *batch, uint32_t world, uint32_t *pairs, uint32_t capacity,
                                   uint32_t *count);
pe_status pe_batch_get_world_contacts(pe_batch *batch, uint32_t world, pe_contact_manifold *out, uint32_t capacity,
                                      uint32_t *count);
pe_status pe_batch_get_stream(pe_batch *batch, void **stream);
pe_status pe_batch_set_graphs(pe_batch *batch, int enabled);

/* ------------------------------------------------------------------------
   Differentiable batched rollout (no reference counterpart; the reference has
   no differentiation).  Many independent worlds of sphere/box bodies (1 to
   8192 per world, one collider each) are stepped `steps` times with
   PhysicsWorld::step's algorithm (SAP pair set, graph-colour solve order) on
   the GPU; the adjoint returns the gradients of sum(d_final . final state)
   with respect to the initial state and to each body's mass (the RigidBody
   field; the inverse inertia stays as created), friction and restitution.
   The contact set of the forward pass is frozen in the adjoint (pairs, kept
   contact features, colour order, warm-start matches, clamp branches); contact
   points, normals and depths are differentiated as functions of the poses.
   Memory: states are checkpointed every `checkpoint_every` steps and each
   segment is recomputed once during the adjoint; each world's device slot
   (checkpoints, one segment's step scratch and tape, adjoints) is sized by its
   own body count, and pe_rollout_device_bytes reports the total.
   State arrays are DEVICE pointers holding all worlds' bodies back to back:
   positions / linear / angular velocities 3 floats per body, rotations 4
   (x, y, z, w).  Calls run on `stream` and return when the work is done.
   ------------------------------------------------------------------------ */
typedef struct pe_rollout pe_rollout;

/* dims / density / is_static as pe_world_create_bodies; mass_out (host, may be
   NULL) receives the created masses (volume x density). */
pe_status pe_rollout_create(int device, uint32_t world_count, const uint32_t *world_body_counts,
                            const uint8_t *shape, const float *dims, const float *density, const uint8_t *is_static,
                            uint32_t steps, float dt, int iterations, uint32_t checkpoint_every, pe_rollout **out,
                            float *mass_out);
void pe_rollout_destroy(pe_rollout *rollout);
pe_status pe_rollout_set_gravity(pe_rollout *rollout, float x, float y, float z);
pe_status pe_rollout_forward(pe_rollout *rollout, const float *x0, const float *q0, const float *v0,
                             const float *w0, const float *mass, const float *friction, const float *restitution,
                             float *x_final, float *q_final, float *v_final, float *w_final, void *stream);
/* Adjoint of the last forward call; any d_final_* input or output may be NULL. */
pe_status pe_rollout_backward(pe_rollout *rollout, const float *d_final_x, const float *d_final_q,
                              const float *d_final_v, const float *d_final_w, float *d_x0, float *d_q0,
                              float *d_v0, float *d_w0, float *d_mass, float *d_friction, float *d_restitution,
                              void *stream);
/* Device time of the last forward and backward calls (ms). */
pe_status pe_rollout_timings(pe_rollout *rollout, double *forward_ms, double *backward_ms);
/* Contact-manifold capacity per body of every world (0.25 to 64; default 2,
   enough for boxes resting on one another).  The device slots are laid out at
   the next forward call; a world whose manifolds outgrow it fails that call. */
pe_status pe_rollout_set_manifold_capacity(pe_rollout *rollout, float per_body);
/* Device memory the rollout holds (bytes; 0 before the first forward call). */
pe_status pe_rollout_device_bytes(pe_rollout *rollout, uint64_t *bytes);

/* Failure detection, for tests (no reference counterpart).  Every spin-wait of
   the step kernels (tile look-back, grid barrier, union retries, colouring
   passes) is bounded by `limit` iterations on `device` (0 = the default,
   2^24).  A wait that runs out makes its kernel return at once and the step
   fail with PE_ERR_DEVICE ("a bounded wait timed out"); the world keeps the
   state it had before that step. */
pe_status pe_debug_set_spin_limit(int device, uint32_t limit);

/* Allocation-free sweep-and-prune query.  It has no counterpart in the
   reference: it exists for callers that may not allocate device memory at all
   (an engine that gives this library a fixed slice of its own memory arena, a
   frame loop in which cudaMalloc's implicit synchronisation breaks the time
   budget, a process that already holds nearly all of the GPU's memory).
   Inputs and outputs are DEVICE pointers owned by the caller: d_mins/d_maxs
   are n xyz triples, d_pairs receives up to `capacity` pairs (2 indices each,
   first < second, in the same lexicographic order as pe_broadphase_find_pairs
   with PE_BROADPHASE_SAP, which it equals), d_result receives two uint32
   words: the number of pairs found, then 0 = all written, 1 = more pairs than
   `capacity` (the first `capacity` written), 2 = more than
   PE_NOALLOC_MAX_PAIRS (nothing written).  The call only enqueues one kernel on
   `stream` (a cudaStream_t; NULL = default stream) and returns; results are
   ready when the stream reaches that point.
   Scratch is a fixed 557,056-byte device array inside the library, present on
   every GPU that loads the library until the process exits; the call makes no
   allocation.  n > PE_NOALLOC_MAX_BOXES is rejected with
   PE_ERR_INVALID_ARGUMENT before anything is enqueued.  The first call on each
   device looks up the array's device address (loading the library's device
   code on that GPU if needed); make that first call before any stream capture.
   All calls share the one array: calls whose kernels may overlap on the GPU
   (different streams, or different host threads) race and corrupt each other's
   results, so serialise them, e.g. on one stream.
   Bounds must be finite with min <= max on every axis, the contract of the
   reference's BroadPhase::findCandidatePairs (include/phys/collision/
   broadphase.hpp:47-51); a NaN bound leaves the pair set unspecified.
   The call switches to `device` to enqueue its kernel and puts the caller's
   current device back before it returns (on errors too).  The array's device
   address is looked up once per device and kept: do not call this on a device
   after cudaDeviceReset in the same process. */
#define PE_NOALLOC_MAX_BOXES 8192u
#define PE_NOALLOC_MAX_PAIRS 32768u
pe_status pe_broadphase_find_pairs_noalloc(int device, const float *d_mins, const float *d_maxs, uint32_t n,
                                           uint32_t *d_pairs, uint32_t capacity, uint32_t *d_result,
                                           void *stream);

#ifdef __cplusplus
}
#endif

#endif
